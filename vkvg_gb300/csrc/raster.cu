/*
 * K5 - per-band coverage and compositing on sm_103a.
 *
 * One CTA (16 warps) owns a tile of up to 1024 pixels x 16 sample rows (4
 * pixel rows at 4x MSAA) and walks the frame's draws in submission order.
 * Warp w owns the 64-pixel strip [64w, 64w + 64) of all 16 rows; lane l owns
 * the 32 consecutive samples of row l/2 starting at column 64w + 32(l&1),
 * whose premultiplied RGBA8 values stay in registers for the whole frame.
 * Compact 64 x 16 warp footprints let a warp skip a draw that neither crosses
 * nor covers its strip, which for scribble-like paths is about half of them.
 *
 * Coverage is exact integer arithmetic on the snapped 24.8 vertices: an edge
 * crossing sample row y at x_c adds its direction (+1 downward, -1 upward) to
 * every sample with x < x_c (a sample on the edge counts as if moved by
 * (+e, +e^2), which is the top-left rule).  Summed over a closed polygon this
 * is its winding number; summed over positively oriented triangles it is the
 * number of covering triangles.  Every (primitive, sample row) pair of a
 * draw's band edges is one work item (stroke triangles arrive as their
 * edges, with the edges neighbouring triangles share in opposite directions
 * already cancelled): each edge crossing is computed
 * exactly (an fp32 quotient estimate corrected by one exact remainder test)
 * and its direction is added to a shared-memory counter at the last sample
 * left of the crossing, to the crossing's (row, strip) total, and the strip
 * is flagged.  After one barrier each lane forms the winding entering its
 * run from the strip totals to its right, loads its 32 counters (flagged
 * strips only) and walks its run right to left with one branch-free select
 * per sample.  The fill rule decides how many times vkvg's blend is applied
 * per sample: even-odd -> w & 1 (the stencil-INVERT fan of _poly_fill),
 * non-zero -> w != 0 (glutess' NONZERO tessellation), stroke -> w (each
 * overlapping stroke triangle blends once under pipe_OVER).
 *
 * Counters and flags are double-buffered and strip totals triple-buffered by
 * draw, so one barrier per draw orders everything: warps that finish a
 * draw's blend start accumulating the next draw while others still blend.
 *
 * Blend (src/vkvg_device_internal.c:200-209, ONE / ONE_MINUS_SRC_ALPHA on
 * premultiplied UNORM8): d' = s + floor((d*(255-sa) + 127) / 255) per channel.
 * For a source whose colour bytes do not exceed its alpha (every colour set
 * through the public API) s + t <= 255 and the blend runs on the FMA pipe:
 * floor((d*inv + 127) / 255) = round(d * inv / 255) (no ties, 255 is odd),
 * and with k = round(inv * 2^23 / 255) / 2^23 (error <= 2^-24, far below the
 * 1/510 distance of d*inv/255 from a half-integer) one fmaf of
 * (2^23 + d) * k + (1.5 * 2^23 + s - k * 2^23) leaves s + t in the low byte
 * of the float's bits (checked exhaustively over d, inv and s <= sa).  Other
 * sources and DIFFERENCE use saturating two-channel integer arithmetic.  At
 * the end the tile writes its samples back and the resolved pixels
 * ((sum + S/2) / S) as 128-bit stores.
 */
#include "gb_types.h"
#include "launch.h"
#include "raster_common.cuh"
#include "xdiv.cuh"

#include <cuda_runtime.h>

#include <atomic>

/* Tile geometry of a raster CTA of NW warps: NW strips of 64 pixels, 16
   sample rows.  Shared memory: 2 counter planes, 3 strip-total sets, 2 flag
   sets; then 2 staging buffers for a cell's records (16-byte units), the
   per-warp draw-chunk tables (192 words each), 2 mbarriers and the walk's
   bounds.  The wide form (16 warps, 1024 pixels, one CTA per SM) suits
   surfaces whose draws span most of a tile; the narrow form (4 warps, 256
   pixels, four CTAs per SM) suits small draws and narrow surfaces, where
   the wide form's warps would wait at each draw's barrier with nothing to
   blend; the middle form (8 warps, 512 pixels, two CTAs per SM) sits
   between them for the batch tuner. */
template <int NW> struct XT {
    static constexpr int W         = 64 * NW;
    static constexpr int THREADS   = 32 * NW;
    static constexpr int MINB      = NW >= 16 ? 1 : NW >= 8 ? 2 : NW >= 4 ? 4 : NW >= 2 ? 8 : 16; /* CTAs per SM */
    static constexpr int PLANE     = GB_BAND_ROWS * W; /* one crossing counter per tile sample */
    static constexpr int TOT_ROW   = NW == 1 ? 4 : (NW + 7) / 4 * 4; /* strip totals per row, padded (int4 rows, bank spread) */
    static constexpr int TOT_SET   = GB_BAND_ROWS * TOT_ROW;
    static constexpr int S_TOT     = 2 * PLANE;
    static constexpr int S_FLAG    = S_TOT + 3 * TOT_SET;
    static constexpr int S_WORDS   = S_FLAG + 2 * NW;
    static constexpr int STAGE_CAP = NW >= 8 ? 128 * NW : NW >= 4 ? 480 : NW >= 2 ? 128 : 64; /* units per staging buffer */
    static constexpr int S_STAGE   = (S_WORDS + 3) / 4 * 4;
    static constexpr int S_CUR     = S_STAGE + 2 * STAGE_CAP * 4;
    static constexpr int S_MBAR    = S_CUR + NW * 192;
    static constexpr int S_RG      = S_MBAR + 4;
    /* narrow form: the band's 4 pixel rows of the current gradient source
       image (4x MSAA), staged once per source instead of loaded per sample */
    static constexpr int GC        = NW <= 4 ? 4 * W : 0;
    static constexpr int S_GC      = S_RG + 8;
    static constexpr int SMEM      = (S_GC + GC) * 4;
    static_assert(S_STAGE % 4 == 0 && S_MBAR % 2 == 0, "staging buffers 16-byte, mbarriers 8-byte aligned");
    static_assert(MINB * (SMEM + 1024) <= 232448, "shared memory of the CTAs an SM holds");
};
#define XT_WIDE   16
#define XT_MID    8
#define XT_NARROW 4
#define XT_TINY   2
#define XT_MICRO  1

/* counter (or staged sample) of tile sample p in band row rr: each lane run
   of 32 samples is eight 16-byte slots, rotated by the row and the run's
   half-strip so that the eight lanes of one 128-byte phase hit distinct banks */
template <int NW> __device__ __forceinline__ uint32_t swz(uint32_t rr, uint32_t p) {
    const uint32_t v = ((rr & 3u) << 1) | ((p >> 5) & 1u);
    return rr * XT<NW>::W + (((p >> 2) ^ v) << 2) + (p & 3u);
}

/* The band's active draws, 32 at a time, from its list of active cells
   (positions [i0, iend) of A.alist: cells with records, and the draws that
   act on every band).  Draws before dlo or from dhi on are passed over, and
   so are fill and stroke draws whose edges all lie left of the tile (they
   cross no sample) or all right of it (their closed contours add a net zero
   to every row; tested on surfaces wider than one tile).  Each warp keeps
   the chunk's (kind, lo, hi, src, op, gsrc) in its own table in shared
   memory (ct), amask the active ones not yet taken.  A band whose list
   holds more than half of the draws walks the draws themselves instead
   (dense: positions are draw indices), which saves the list's dependent
   load.  The walk's bounds are CTA-uniform and live in shared memory
   (smem + S_RG), out of the registers the blend needs.  All warps walk the
   same sequence. */
struct draw_cursor {
    uint32_t i0, amask;
};
struct draw_range {
    uint32_t iend, dlo, dhi;
    int32_t  tx_lo, tx_hi;
    uint32_t tiles, dense;
};
template <int NW, bool CLIP>
__device__ __forceinline__ void cur_load(draw_cursor &c, const gb_raster_args &A, size_t cb, const int32_t *smem,
                                         uint32_t l, uint32_t *ct) {
    const draw_range &rg  = *reinterpret_cast<const draw_range *>(smem + XT<NW>::S_RG);
    const uint32_t    il  = c.i0 + l;
    bool              act = false;
    uint32_t          kind = 0, lo = 0, hi = 0, src = 0, op = 0, gs = 0;
    if (il < rg.iend) {
        const uint32_t dl = rg.dense ? il : A.alist[il] - A.cell0 - (uint32_t)cb;
        if (dl >= rg.dlo && dl < rg.dhi) {
            const gb_draw &D = A.draws[dl];
            kind             = D.kind;
            src              = D.src;
            op               = D.op;
            gs               = D.gsrc;
            lo               = A.cell_off[cb + dl];
            hi               = A.cell_off[cb + dl + 1];
            /* paint, clear and the clip kinds act on every band; the others only
               where they have geometry */
            act = kind == GB_DRAW_PAINT || (CLIP ? kind >= GB_DRAW_CLEAR : kind == GB_DRAW_CLEAR) || lo != hi;
            if (rg.tiles && act && kind <= GB_DRAW_STROKE && A.dbox) {
                const int2 bx = A.dbox[dl];
                act           = bx.x <= rg.tx_hi && -bx.y >= rg.tx_lo;
            }
        }
    }
    __syncwarp();
    ct[l]       = kind;
    ct[32 + l]  = lo;
    ct[64 + l]  = hi;
    ct[96 + l]  = src;
    ct[128 + l] = op;
    ct[160 + l] = gs;
    c.amask    = __ballot_sync(0xffffffffu, act);
}
/* the next active draw: its list position (the identity the staging
   buffers use), kind, record range and table slot */
template <int NW, bool CLIP>
__device__ __forceinline__ bool cur_next(draw_cursor &c, const gb_raster_args &A, size_t cb, const int32_t *smem,
                                         uint32_t l, uint32_t *ct, uint32_t *d, uint32_t *kind, uint32_t *lo,
                                         uint32_t *hi, uint32_t *slot) {
    while (c.amask == 0) {
        c.i0 += 32;
        if (c.i0 >= reinterpret_cast<const draw_range *>(smem + XT<NW>::S_RG)->iend)
            return false;
        cur_load<NW, CLIP>(c, A, cb, smem, l, ct);
    }
    const int j = __ffs(c.amask) - 1;
    c.amask &= c.amask - 1;
    *d    = c.i0 + (uint32_t)j;
    *slot = (uint32_t)j;
    *kind = ct[j];
    *lo   = ct[32 + j];
    *hi   = ct[64 + j];
    return true;
}
/* the stencil's save bits of a word go to zero (vkvg_reset_clip / vkvg_clear
   clear the whole stencil attachment) */
__device__ __forceinline__ void clip_zero_planes(uint32_t *cpl, size_t pw) {
#pragma unroll
    for (int p = 0; p < GB_CLIP_SAVE_PLANES; p++)
        cpl[p * pw] = 0u;
}
/* kinds whose records are staged (the variant without clipping sees no clip draws) */
template <bool CLIP> __device__ __forceinline__ bool is_geom(uint32_t kind) {
    if (CLIP)
        return kind <= GB_DRAW_STROKE || kind == GB_DRAW_CLIP_EO || kind == GB_DRAW_CLIP_NZ;
    return kind != GB_DRAW_PAINT && kind != GB_DRAW_CLEAR;
}

/* one edge crossing sample row sy (band row rr): add dir at the last tile
   sample left of the crossing, so that the suffix sum from sample c is the
   winding contribution at c */
template <int NW>
__device__ __forceinline__ void acc_row(int32_t x0, int32_t y0, int32_t x1, int32_t y1, int32_t sy, uint32_t rr,
                                        int32_t ox, int32_t X0, int32_t TW, int32_t tx_lo, int32_t tx_hi,
                                        int32_t *__restrict__ plane, int32_t *__restrict__ tot,
                                        int32_t *__restrict__ flag) {
    const int32_t ylo = min(y0, y1), yhi = max(y0, y1);
    if (sy < ylo || sy >= yhi)
        return; /* also drops horizontal edges */
    if (max(x0, x1) < tx_lo)
        return; /* crossing left of every tile sample */
    const int32_t dir = y0 < y1 ? 1 : -1;
    int32_t       k;
    if (min(x0, x1) > tx_hi) {
        k = TW;
    } else {
        const int32_t   dy  = y1 - y0;
        const int32_t   den = dy < 0 ? -dy : dy;
        const int32_t   dxn = dy < 0 ? x0 - x1 : x1 - x0;
        const long long c   = gb_ceil_muldiv(dxn, sy - y0, den);
        const long long kt  = (((long long)x0 + c - 1 - ox) >> 8) + 1 - X0; /* tile samples left of crossing */
        if (kt <= 0)
            return;
        k = kt > TW ? TW : (int32_t)kt;
    }
    const uint32_t p = (uint32_t)(k - 1);
    atomicAdd(&plane[swz<NW>(rr, p)], dir);
    atomicAdd(&tot[rr * XT<NW>::TOT_ROW + (p >> 6)], dir);
    flag[p >> 6] = 1;
}

/* row y of gradient source image gs - 1, from column x */
__device__ __forceinline__ const uint32_t *grad_row(const gb_raster_args &A, uint32_t gs, uint32_t y, int32_t x) {
    return A.gsrc + ((size_t)(gs - 1) * A.H + y) * A.W + x;
}
__device__ __forceinline__ void load_src4(const uint32_t *row, int c0, int ncols, uint32_t (&s)[4]) {
#pragma unroll
    for (int k = 0; k < 4; k++)
        s[k] = c0 + k < ncols ? row[c0 + k] : 0u;
}
/* one sample's blend: the draw's solid source (mode M, constants B) or, for
   G, the sample's own gradient source word s */
template <int M, bool G> __device__ __forceinline__ uint32_t blend_any(uint32_t d, const blend_k &B, uint32_t s) {
    if (G)
        return blend_src(d, s);
    return blend<M>(d, B);
}
/* blend group q of a run where p_k is set */
template <int M, bool G>
__device__ __forceinline__ void blend_group(uint32_t (&col)[32], int q, bool p0, bool p1, bool p2, bool p3,
                                            const blend_k &B, const uint32_t *row, int ncols) {
    uint32_t sv[4] = {0u, 0u, 0u, 0u};
    if (G)
        load_src4(row, 4 * q, ncols, sv);
    const uint32_t n3 = blend_any<M, G>(col[4 * q + 3], B, sv[3]), n2 = blend_any<M, G>(col[4 * q + 2], B, sv[2]);
    const uint32_t n1 = blend_any<M, G>(col[4 * q + 1], B, sv[1]), n0 = blend_any<M, G>(col[4 * q], B, sv[0]);
    col[4 * q + 3]    = p3 ? n3 : col[4 * q + 3];
    col[4 * q + 2]    = p2 ? n2 : col[4 * q + 2];
    col[4 * q + 1]    = p1 ? n1 : col[4 * q + 1];
    col[4 * q]        = p0 ? n0 : col[4 * q];
}

/* Runs with crossings (counters at cp, slot rotation v), right to left in
   groups of four samples; a group is skipped when no lane of the warp has a
   sample to blend in it (about three groups in ten of a mixed warp for
   scribble-like paths), which the vote decides for the whole warp.  Fills
   blend where (w & fmask) != 0 (fmask 1: even-odd, ~0: non-zero); with CL,
   only samples whose bit of the clip word cm is set. */
template <int M, bool G, bool CL>
__device__ __forceinline__ void fill_run(uint32_t (&col)[32], const int4 *cp, uint32_t v, int32_t E, int32_t fmask,
                                         const blend_k &B, const uint32_t *row, int ncols, uint32_t cm) {
    int32_t w = E;
#pragma unroll
    for (int q = 7; q >= 0; q--) {
        const int4    x  = cp[q ^ v];
        const int32_t w3 = w + x.w, w2 = w3 + x.z, w1 = w2 + x.y, w0 = w1 + x.x;
        bool          p3 = (w3 & fmask) != 0, p2 = (w2 & fmask) != 0, p1 = (w1 & fmask) != 0, p0 = (w0 & fmask) != 0;
        if (CL) {
            const uint32_t g = cm >> (4 * q);
            p0 = p0 && (g & 1u), p1 = p1 && (g & 2u), p2 = p2 && (g & 4u), p3 = p3 && (g & 8u);
        }
        w = w0;
        if (__any_sync(0xffffffffu, p0 | p1 | p2 | p3))
            blend_group<M, G>(col, q, p0, p1, p2, p3, B, row, ncols);
    }
}
/* strokes: blend w times (w = covering triangles), one pass per blend; the
   number of passes is the warp's largest w, so that every lane takes part in
   every vote */
template <int M, bool G, bool CL>
__device__ __forceinline__ void stroke_run(uint32_t (&col)[32], const int4 *cp, uint32_t v, int32_t E,
                                           const blend_k &B, const uint32_t *row, int ncols, uint32_t cm) {
    int32_t kmax = 1, kwarp = 1;
    for (int32_t rep = 0; rep < kwarp; rep++) {
        int32_t w = E;
#pragma unroll
        for (int q = 7; q >= 0; q--) {
            const int4    x  = cp[q ^ v];
            const int32_t w3 = w + x.w, w2 = w3 + x.z, w1 = w2 + x.y, w0 = w1 + x.x;
            w                = w0;
            kmax             = max(kmax, max(max(w3, w2), max(w1, w0)));
            bool p3 = w3 > rep, p2 = w2 > rep, p1 = w1 > rep, p0 = w0 > rep;
            if (CL) {
                const uint32_t g = cm >> (4 * q);
                p0 = p0 && (g & 1u), p1 = p1 && (g & 2u), p2 = p2 && (g & 4u), p3 = p3 && (g & 8u);
            }
            if (__any_sync(0xffffffffu, p0 | p1 | p2 | p3))
                blend_group<M, G>(col, q, p0, p1, p2, p3, B, row, ncols);
        }
        if (rep == 0)
            kwarp = __reduce_max_sync(0xffffffffu, kmax);
    }
}
/* a run without crossings: blend every sample (with CL, every sample inside
   the clip) k times */
template <int M, bool G, bool CL>
__device__ __forceinline__ void uniform_run(uint32_t (&col)[32], int32_t k, const blend_k &B, const uint32_t *row,
                                            int ncols, uint32_t cm) {
    for (int32_t rep = 0; rep < k; rep++) {
#pragma unroll
        for (int q = 0; q < 8; q++) {
            uint32_t sv[4] = {0u, 0u, 0u, 0u};
            if (G)
                load_src4(row, 4 * q, ncols, sv);
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int      c  = 4 * q + e;
                const uint32_t nb = blend_any<M, G>(col[c], B, sv[e]);
                col[c]            = (!CL || ((cm >> c) & 1u)) ? nb : col[c];
            }
        }
    }
}
/* a clip draw on a run with crossings: the bits of the samples it covers */
__device__ __forceinline__ uint32_t clip_bits(const int4 *cp, uint32_t v, int32_t E, int32_t fmask) {
    int32_t  w    = E;
    uint32_t bits = 0;
#pragma unroll
    for (int q = 7; q >= 0; q--) {
        const int4    x  = cp[q ^ v];
        const int32_t w3 = w + x.w, w2 = w3 + x.z, w1 = w2 + x.y, w0 = w1 + x.x;
        bits |= ((w0 & fmask) ? 1u : 0u) << (4 * q) | ((w1 & fmask) ? 2u : 0u) << (4 * q) |
                ((w2 & fmask) ? 4u : 0u) << (4 * q) | ((w3 & fmask) ? 8u : 0u) << (4 * q);
        w = w0;
    }
    return bits;
}

/* One cell of the raster: sample rows [16 band, 16 band + 16) and columns
   [W tile, W tile + W) of A's surface (W = 64 NW), through every draw of the
   surface in order, then the resolve of its pixels. */
template <int NW, bool GRAD, bool CLIP>
__device__ __forceinline__ void raster_item(const gb_raster_args &A, const gb_clip_args &C, int32_t *smem,
                                            uint32_t band, uint32_t tile) {
    using X          = XT<NW>;
    const uint32_t t = threadIdx.x, wi = t >> 5, l = t & 31;
    const uint32_t rl = l >> 1, hh = l & 1; /* blend mapping: band row and half-strip */
    const int32_t  X0      = (int32_t)(tile * X::W);
    const int32_t  TW      = min((int32_t)X::W, (int32_t)A.W - X0);
    const int32_t  R       = (int32_t)(band * GB_BAND_ROWS + rl);
    const bool     row_ok  = R < (int32_t)A.nrows;
    const int32_t  col0    = (int32_t)(64 * wi + 32 * hh);
    const int32_t  ncols   = row_ok ? max(0, min(32, TW - col0)) : 0;
    const int32_t  band_r0 = (int32_t)(band * GB_BAND_ROWS);
    const int32_t  tx_lo = X0 * 256 + 32, tx_hi = (X0 + TW - 1) * 256 + 224;
    const uint32_t nd      = A.ndraws;
    const size_t   cb      = (size_t)band * nd;
    const bool     dbg     = A.cov_out != nullptr;
    const uint32_t rpp     = A.S == 4 ? 4 : 1;
    const uint32_t v_lane  = ((rl & 3u) << 1) | hh; /* slot rotation of this lane's run */
    /* accumulate mapping: item rows (rr = t & 15) */
    const uint32_t irr = t & 15;
    const int32_t  iR  = band_r0 + (int32_t)irr;
    const bool     iok = iR < (int32_t)A.nrows;
    const int32_t  isy = A.S == 4 ? 32 + 64 * iR : 128 + 256 * iR;
    const int32_t  iox = A.S == 4 ? ((iR & 3) == 0 ? 96 : (iR & 3) == 1 ? 224 : (iR & 3) == 2 ? 32 : 160) : 128;

    uint32_t  col[32];
    uint32_t *srow = A.samples + (size_t)(row_ok ? R : 0) * A.Wpad + X0 + col0;
    if (A.init_mode == 1) {
#pragma unroll
        for (int c = 0; c < 32; c++)
            col[c] = A.init_color;
    } else if (ncols == 32) {
        const uint4 *p = reinterpret_cast<const uint4 *>(srow);
#pragma unroll
        for (int q = 0; q < 8; q++) {
            uint4 v        = p[q];
            col[4 * q]     = v.x;
            col[4 * q + 1] = v.y;
            col[4 * q + 2] = v.z;
            col[4 * q + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int c = 0; c < 32; c++)
            col[c] = c < ncols ? srow[c] : 0u;
    }
    /* this lane's clip word: one bit per sample of its run */
    const size_t cwi = (size_t)(row_ok ? R : 0) * C.clip_wpr + (uint32_t)(X0 + col0) / 32u;
    uint32_t     cm  = 0xFFFFFFFFu;
    /* live save planes of this lane's word: plane p at cpl[p * plane_words] */
    uint32_t *const cpl = CLIP ? C.clip_planes + cwi : nullptr;
    const bool      cwr = CLIP && row_ok && ncols > 0; /* this lane owns a clip word */
    if (CLIP && C.clip_load == 1 && ncols > 0)
        cm = C.clip[cwi];
    if (CLIP && C.clip_load == 2 && cwr && !dbg)
        clip_zero_planes(cpl, C.plane_words);
    for (uint32_t i = t; i < X::S_WORDS; i += X::THREADS)
        smem[i] = 0;
    const uint32_t sm_base = (uint32_t)__cvta_generic_to_shared(smem);
    const uint32_t bar0    = sm_base + X::S_MBAR * 4;
    if (t == 0) {
        mbar_init(bar0);
        mbar_init(bar0 + 8);
        mbar_init_fence();
        draw_range &rg = *reinterpret_cast<draw_range *>(smem + X::S_RG);
        const uint32_t ib = A.apos[cb], ie = A.apos[cb + nd];
        rg.dlo            = dbg ? A.cov_draw : A.draw_first;
        rg.dhi            = dbg ? A.cov_draw + 1 : nd;
        rg.dense          = 2u * (ie - ib) > nd ? 1u : 0u;
        rg.iend           = rg.dense ? rg.dhi : ie;
        rg.tx_lo          = tx_lo;
        rg.tx_hi          = tx_hi;
        rg.tiles          = A.W > X::W ? 1u : 0u;
        smem[X::S_RG + 7] = rg.dense ? rg.dlo : ib; /* the walk's first position */
    }
    __syncthreads();
    /* staging state, identical in every thread: the draw each buffer holds
       or receives, the parity its mbarrier completes next, copies not yet
       seen to complete */
    uint32_t stg_d0 = 0xFFFFFFFFu, stg_d1 = 0xFFFFFFFFu;
    uint32_t stg_par = 0, stg_pend = 0;
    auto     stage_cell = [&](uint32_t b, uint32_t d, uint32_t lo, uint32_t units) {
        if (t == 0)
            stage_copy(sm_base + (X::S_STAGE + b * X::STAGE_CAP * 4) * 4, A.recs + lo, units * 16u, bar0 + 8 * b);
        if (b)
            stg_d1 = d;
        else
            stg_d0 = d;
        stg_pend |= 1u << b;
    };

    uint32_t    nproc = 0; /* draws with geometry in this band so far */
    /* gradient rows staged in shared memory (narrow form, 4x MSAA): which
       source they hold, and this lane's row of them */
    const bool      gc_on  = GRAD && X::GC > 0 && A.S == 4 && !dbg;
    uint32_t        gc_gs  = 0;
    const uint32_t *gc_row = reinterpret_cast<const uint32_t *>(smem + X::S_GC) + (rl >> 2) * X::W + col0;
    uint32_t   *ct    = reinterpret_cast<uint32_t *>(smem + X::S_CUR + wi * 192);
    draw_cursor cur;
    cur.i0 = (uint32_t)smem[X::S_RG + 7];
    cur_load<NW, CLIP>(cur, A, cb, smem, l, ct);
    uint32_t nx_d = 0, nx_kind = 0, nx_lo = 0, nx_hi = 0, nx_slot = 0;
    bool     nx_have = cur_next<NW, CLIP>(cur, A, cb, smem, l, ct, &nx_d, &nx_kind, &nx_lo, &nx_hi, &nx_slot);
    {
        while (nx_have) {
            const uint32_t d = nx_d, kind = nx_kind, lo = nx_lo, hi = nx_hi;
            const uint32_t src = ct[96 + nx_slot], op = ct[128 + nx_slot], gs = ct[160 + nx_slot];
            nx_have = cur_next<NW, CLIP>(cur, A, cb, smem, l, ct, &nx_d, &nx_kind, &nx_lo, &nx_hi, &nx_slot); /* lookahead */
            if (gc_on && gs && gs != gc_gs) {
                /* a new gradient source: once every warp is done with the
                   old rows, the tile's pixel rows of this one */
                __syncthreads();
                uint32_t *gc = reinterpret_cast<uint32_t *>(smem + X::S_GC);
                for (uint32_t i = t; i < (uint32_t)X::GC; i += X::THREADS) {
                    const uint32_t pr = i / X::W, px = i % X::W, py = band * 4 + pr;
                    gc[i] = ((int32_t)px < TW && py < A.H) ? grad_row(A, gs, py, X0 + (int32_t)px)[0] : 0u;
                }
                __syncthreads();
                gc_gs = gs;
            }
            int            bm;
            if (kind == GB_DRAW_PAINT) {
                const blend_k B = make_blend(src, op, &bm);
                if (dbg) {
                    for (int c = 0; c < ncols; c++)
                        A.cov_out[((size_t)(R / rpp) * A.W + X0 + col0 + c) * A.S + R % rpp] = 1;
                    continue;
                }
                if (GRAD && gs)
                    uniform_run<BM_ADD, GRAD, CLIP>(col, 1, B, gc_on ? gc_row : grad_row(A, gs, R / rpp, X0 + col0),
                                                    ncols, cm);
                else if (bm == BM_ADD)
                    uniform_run<BM_ADD, false, CLIP>(col, 1, B, nullptr, ncols, cm);
                else if (bm == BM_SADD)
                    uniform_run<BM_SADD, false, CLIP>(col, 1, B, nullptr, ncols, cm);
                else
                    uniform_run<BM_SSUB, false, CLIP>(col, 1, B, nullptr, ncols, cm);
                continue;
            }
            if (kind == GB_DRAW_CLEAR) { /* colour and the whole stencil: clip and save planes */
#pragma unroll
                for (int c = 0; c < 32; c++)
                    col[c] = 0u;
                cm = 0xFFFFFFFFu;
                if (CLIP && cwr && !dbg)
                    clip_zero_planes(cpl, C.plane_words);
                continue;
            }
            if (CLIP && kind >= GB_DRAW_CLIP_RESET) { /* stencil plane operations, parameter in src */
                if (CLIP && cwr && !dbg) {
                    const size_t pw = C.plane_words;
                    if (kind == GB_DRAW_CLIP_RESET) {
                        cm = 0xFFFFFFFFu;
                        clip_zero_planes(cpl, pw);
                    } else if (kind == GB_DRAW_CLIP_SAVE) {
                        cpl[src * pw] = ~cm;
                    } else if (kind == GB_DRAW_CLIP_RESTORE) {
                        cm = ~cpl[src * pw];
                    } else {
                        uint32_t *img = cpl + (size_t)(GB_CLIP_SAVE_PLANES + GB_CLIP_IMAGE_PLANES * src) * pw;
                        if (kind == GB_DRAW_CLIP_STORE) {
                            img[0] = cm;
#pragma unroll
                            for (int p = 0; p < GB_CLIP_SAVE_PLANES; p++)
                                img[(1 + p) * pw] = cpl[p * pw];
                        } else {
                            cm = img[0];
#pragma unroll
                            for (int p = 0; p < GB_CLIP_SAVE_PLANES; p++)
                                cpl[p * pw] = img[(1 + p) * pw];
                        }
                    }
                }
                continue;
            }
            /* clip draws reach only the clipping variant */
            const bool is_clip = CLIP && (kind == GB_DRAW_CLIP_EO || kind == GB_DRAW_CLIP_NZ);
            if (is_clip && lo == hi) { /* the clip path has nothing in this band */
                if (CLIP && !dbg)
                    cm = 0u;
                continue;
            }
            if (hi > A.nunits || lo > hi) {
                if (t == 0)
                    atomicOr(A.status, GB_ERR_OVERFLOW);
                continue;
            }
            const blend_k B = make_blend(src, op, &bm);
            /* this draw's records: staged now unless prefetched; then prefetch
               the next geometry draw into the other buffer, whose readers all
               passed the previous barrier */
            /* cells below stage_min units are read from global memory by
               the accumulating threads instead (the same test decides the
               prefetch, so every copy issued is waited for) */
            const uint32_t sb  = nproc & 1;
            const bool     stg = hi - lo >= A.stage_min;
            const uint32_t su  = stg ? min(hi - lo, (uint32_t)X::STAGE_CAP) : 0u;
            if (stg && (sb ? stg_d1 : stg_d0) != d)
                stage_cell(sb, d, lo, su);
            if (nx_have && is_geom<CLIP>(nx_kind) && nx_lo < nx_hi && nx_hi <= A.nunits &&
                nx_hi - nx_lo >= A.stage_min)
                stage_cell(sb ^ 1u, nx_d, nx_lo, min(nx_hi - nx_lo, (uint32_t)X::STAGE_CAP));
            if (stg) {
                if (mbar_wait(bar0 + 8 * sb, (stg_par >> sb) & 1u)) {
                    stg_pend &= ~(1u << sb);
                } else if (t == 0) {
                    atomicOr(A.status, GB_ERR_RASTER_WAIT);
                }
                stg_par ^= 1u << sb;
                if (sb)
                    stg_d1 = 0xFFFFFFFFu;
                else
                    stg_d0 = 0xFFFFFFFFu;
            }
            const int4 *sg = reinterpret_cast<const int4 *>(smem + X::S_STAGE) + sb * X::STAGE_CAP;
            int32_t *plane = smem + (nproc & 1) * X::PLANE;
            int32_t *tot   = smem + X::S_TOT + (nproc % 3) * X::TOT_SET;
            int32_t *flag  = smem + X::S_FLAG + (nproc & 1) * NW;

            /* ---- accumulate: one item per (primitive, band row) */
            if (iok) {
                const uint32_t n = (hi - lo) * 16u;
                for (uint32_t it = t; it < n; it += X::THREADS) {
                    const uint32_t u  = it >> 4;
                    const int4     ed = u < su ? sg[u] : A.recs[lo + u];
                    acc_row<NW>(ed.x, ed.y, ed.z, ed.w, isy, irr, iox, X0, TW, tx_lo, tx_hi, plane, tot, flag);
                }
            }
            __syncthreads();

            /* ---- blend.  The previous draw's totals are no longer read by anyone. */
            if (hh == 0)
                smem[X::S_TOT + ((nproc + 2) % 3) * X::TOT_SET + rl * X::TOT_ROW + wi] = 0;
            nproc++;
            int32_t Er = 0; /* winding from strips to the right */
            {
                const int4 *tr4 = reinterpret_cast<const int4 *>(tot + rl * X::TOT_ROW);
#pragma unroll
                for (int q = 0; q < (NW + 3) / 4; q++) {
                    const int4 v = tr4[q];
                    Er += (4 * q > (int)wi ? v.x : 0) + (4 * q + 1 > (int)wi ? v.y : 0) +
                          (4 * q + 2 > (int)wi ? v.z : 0) + (4 * q + 3 > (int)wi ? v.w : 0);
                }
            }
            const bool flagged = flag[wi] != 0;

            if (dbg) {
                /* coverage of a single draw: read the counters in place */
                int32_t L = 0;
                for (int c = 0; c < 32; c++)
                    L += plane[swz<NW>(rl, col0 + c)];
                const int32_t Lp = __shfl_xor_sync(0xffffffffu, L, 1);
                int32_t       w  = Er + (hh == 0 ? Lp : 0);
                for (int c = 31; c >= 0; c--) {
                    w += plane[swz<NW>(rl, col0 + c)];
                    if (c < ncols)
                        A.cov_out[((size_t)(R / rpp) * A.W + X0 + col0 + c) * A.S + R % rpp] = w;
                }
                continue;
            }
            if (!flagged) {
                /* no crossing in the strip: every run has the uniform winding Er */
                int32_t k = 0;
                if (row_ok)
                    k = kind == GB_DRAW_STROKE                                             ? max(Er, 0)
                        : (kind == GB_DRAW_FILL_EO || (CLIP && kind == GB_DRAW_CLIP_EO)) ? (Er & 1)
                                                                                         : (Er != 0);
                if (is_clip) { /* the whole run is inside the clip path or outside it */
                    if (CLIP && !k)
                        cm = 0u;
                    continue;
                }
                if (!__any_sync(0xffffffffu, k > 0))
                    continue;
                if (GRAD && gs)
                    uniform_run<BM_ADD, GRAD, CLIP>(col, k, B, gc_on ? gc_row : grad_row(A, gs, R / rpp, X0 + col0),
                                                    ncols, cm);
                else if (bm == BM_ADD)
                    uniform_run<BM_ADD, false, CLIP>(col, k, B, nullptr, ncols, cm);
                else if (bm == BM_SADD)
                    uniform_run<BM_SADD, false, CLIP>(col, k, B, nullptr, ncols, cm);
                else
                    uniform_run<BM_SSUB, false, CLIP>(col, k, B, nullptr, ncols, cm);
                continue;
            }
            /* this lane's 32 counters: totals first, the blend reads them again;
               then they are cleared for the draw after next */
            int4   *cp  = reinterpret_cast<int4 *>(plane + rl * X::W + col0);
            int     nzr = 0;
            int32_t L   = 0;
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int4 x = cp[q ^ v_lane];
                nzr |= x.x | x.y | x.z | x.w;
                L += x.x + x.y + x.z + x.w;
            }
            const int32_t Lp   = __shfl_xor_sync(0xffffffffu, L, 1);
            const int32_t E    = Er + (hh == 0 ? Lp : 0); /* winding entering this run from the right */
            const bool    work = row_ok && (nzr != 0 || E != 0);
            if (is_clip) { /* the clip region keeps the samples the path covers */
                if (CLIP)
                    cm &= clip_bits(cp, v_lane, E, kind == GB_DRAW_CLIP_EO ? 1 : -1);
            } else if (__any_sync(0xffffffffu, work)) {
                const int32_t fmask = kind == GB_DRAW_FILL_EO ? 1 : -1;
                if (GRAD && gs) {
                    const uint32_t *grow = gc_on ? gc_row : grad_row(A, gs, R / rpp, X0 + col0);
                    if (kind == GB_DRAW_STROKE)
                        stroke_run<BM_ADD, GRAD, CLIP>(col, cp, v_lane, E, B, grow, ncols, cm);
                    else
                        fill_run<BM_ADD, GRAD, CLIP>(col, cp, v_lane, E, fmask, B, grow, ncols, cm);
                } else if (kind == GB_DRAW_STROKE) {
                    if (bm == BM_ADD)
                        stroke_run<BM_ADD, false, CLIP>(col, cp, v_lane, E, B, nullptr, ncols, cm);
                    else if (bm == BM_SADD)
                        stroke_run<BM_SADD, false, CLIP>(col, cp, v_lane, E, B, nullptr, ncols, cm);
                    else
                        stroke_run<BM_SSUB, false, CLIP>(col, cp, v_lane, E, B, nullptr, ncols, cm);
                } else {
                    if (bm == BM_ADD)
                        fill_run<BM_ADD, false, CLIP>(col, cp, v_lane, E, fmask, B, nullptr, ncols, cm);
                    else if (bm == BM_SADD)
                        fill_run<BM_SADD, false, CLIP>(col, cp, v_lane, E, fmask, B, nullptr, ncols, cm);
                    else
                        fill_run<BM_SSUB, false, CLIP>(col, cp, v_lane, E, fmask, B, nullptr, ncols, cm);
                }
            }
#pragma unroll
            for (int q = 0; q < 8; q++)
                cp[q ^ v_lane] = make_int4(0, 0, 0, 0);
            __syncwarp();
            if (l == 0)
                flag[wi] = 0;
        }
    }
    /* a copy that missed its wait limit may still land: wait for it (again
       bounded) before the shared memory is reused or released */
    for (uint32_t b = 0; b < 2; b++)
        if ((stg_pend >> b) & 1u)
            mbar_wait(bar0 + 8 * b, ((stg_par >> b) & 1u) ^ 1u);
    if (dbg)
        return;
    if (cwr)
        C.clip[cwi] = cm;

    /* write back samples */
    if (ncols == 32) {
        uint4 *p = reinterpret_cast<uint4 *>(srow);
#pragma unroll
        for (int q = 0; q < 8; q++)
            p[q] = make_uint4(col[4 * q], col[4 * q + 1], col[4 * q + 2], col[4 * q + 3]);
    } else {
#pragma unroll
        for (int c = 0; c < 32; c++)
            if (c < ncols)
                srow[c] = col[c];
    }
    /* resolve through shared memory (aliases the counter planes); lanes
       stage their runs in the counters' rotated slot order */
    __syncthreads();
    uint4 *stage4 = reinterpret_cast<uint4 *>(smem + rl * X::W + col0);
#pragma unroll
    for (int q = 0; q < 8; q++)
        stage4[q ^ v_lane] = make_uint4(col[4 * q], col[4 * q + 1], col[4 * q + 2], col[4 * q + 3]);
    __syncthreads();
    const uint32_t *stage = reinterpret_cast<const uint32_t *>(smem);
    const uint32_t  prows = GB_BAND_ROWS / rpp;
    const uint32_t  npx   = prows * X::W;
    for (uint32_t q = t * 4; q < npx; q += X::THREADS * 4) {
        uint32_t pr = q / X::W, px = q % X::W; /* 4 consecutive pixels px..px+3 */
        uint32_t py = band * prows + pr;
        if (py >= A.H || (int32_t)px >= TW)
            continue;
        uint32_t outp[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            uint32_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
            for (uint32_t s = 0; s < rpp; s++) {
                uint32_t v = stage[swz<NW>(pr * rpp + s, px + k)];
                s0 += v & 0xFFu;
                s1 += (v >> 8) & 0xFFu;
                s2 += (v >> 16) & 0xFFu;
                s3 += v >> 24;
            }
            uint32_t h = rpp / 2;
            outp[k]    = ((s0 + h) / rpp) | (((s1 + h) / rpp) << 8) | (((s2 + h) / rpp) << 16) | (((s3 + h) / rpp) << 24);
        }
        uint32_t *dst = A.rgba + (size_t)py * A.W + X0 + px;
        if ((int32_t)px + 4 <= TW && ((((uintptr_t)dst) & 15u) == 0)) {
            *reinterpret_cast<uint4 *>(dst) = make_uint4(outp[0], outp[1], outp[2], outp[3]);
        } else {
            for (int k = 0; k < 4; k++)
                if ((int32_t)(px + k) < TW)
                    dst[k] = outp[k];
        }
    }
}

template <int NW, bool GRAD, bool CLIP>
__global__ void __launch_bounds__(XT<NW>::THREADS, XT<NW>::MINB) gb_raster(gb_raster_args A, gb_clip_args C) {
    extern __shared__ __align__(16) int32_t smem[];
    raster_item<NW, GRAD, CLIP>(A, C, smem, blockIdx.y, blockIdx.x);
}

__device__ __forceinline__ void mbar_inval(uint32_t bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
}
/* The batch raster: a persistent grid (one CTA per SM) takes (surface, band,
   tile) items from the work list in queue order until it is exhausted (no
   wait on other CTAs: each CTA stops at the end of the list).  An item's
   arguments are its surface's entry of the table over A0's shared fields,
   staged in shared memory for the whole CTA. */
template <int NW, bool GRAD>
__global__ void __launch_bounds__(XT<NW>::THREADS, XT<NW>::MINB)
    gb_raster_batch(gb_raster_args A0, const gb_surf *__restrict__ surfs, const uint4 *__restrict__ items,
                    uint32_t nitems, uint32_t *__restrict__ queue) {
    extern __shared__ __align__(16) int32_t smem[];
    __shared__ gb_raster_args Ai;
    __shared__ uint32_t       cur_item, cur_band, cur_tile;
    const gb_clip_args        C0 = {};
    for (uint32_t iter = 0; iter < nitems; iter++) {
        if (threadIdx.x == 0) {
            const uint32_t it = atomicAdd(queue, 1u);
            cur_item          = it;
            if (it < nitems) {
                const uint4    w  = items[it];
                const gb_surf &sf = surfs[w.x];
                gb_raster_args a  = A0;
                a.W               = sf.W;
                a.H               = sf.H;
                a.Wpad            = sf.wpad;
                a.nrows           = sf.nrows;
                a.nbands          = sf.nbands;
                a.ndraws          = sf.ndraws;
                a.draw_first      = sf.draw_first;
                a.init_mode       = sf.init_mode;
                a.init_color      = sf.init_color;
                a.draws           = A0.draws + sf.draw0;
                a.cell_off        = A0.cell_off + sf.cell0;
                a.apos            = A0.apos + sf.cell0;
                a.cell0           = (uint32_t)sf.cell0;
                a.dbox            = A0.dbox ? A0.dbox + sf.draw0 : nullptr;
                a.samples         = sf.samples;
                a.rgba            = sf.rgba;
                a.gsrc            = sf.gsrc;
                Ai                = a;
                cur_band          = w.y;
                cur_tile          = w.z;
            }
        }
        __syncthreads();
        if (cur_item >= nitems)
            break;
        raster_item<NW, GRAD, false>(Ai, C0, smem, cur_band, cur_tile);
        __syncthreads();
        if (threadIdx.x == 0) { /* the next item initialises them again */
            const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(smem) + XT<NW>::S_MBAR * 4;
            mbar_inval(bar0);
            mbar_inval(bar0 + 8);
        }
    }
}

/* ---- linear gradient sources.
 *
 * vkvg evaluates the gradient per fragment at the pixel centre
 * (shaders/vkvg_main.frag:83-108): positions normalised by the surface size,
 * the signed distance of the pixel along the gradient axis in units of its
 * length, then the stop colours combined with GLSL's mix and smoothstep, the
 * result times the draw's opacity written to the UNORM8 target.  The
 * expression is evaluated here in that order with explicitly rounded IEEE
 * fp32 operations (no contraction), exactly as the CPU restatement does, and
 * quantised to 8 bits by round-to-nearest; rounding is monotonic, so every
 * colour byte stays at or below the alpha byte of the premultiplied result. */
__device__ __forceinline__ float g_smoothstep(float e0, float e1, float x) {
    float t = __fdiv_rn(__fsub_rn(x, e0), __fsub_rn(e1, e0));
    t       = fminf(fmaxf(t, 0.0f), 1.0f);
    return __fmul_rn(__fmul_rn(t, t), __fsub_rn(3.0f, __fmul_rn(2.0f, t)));
}
__device__ __forceinline__ float g_mix(float x, float y, float a) {
    return __fadd_rn(__fmul_rn(x, __fsub_rn(1.0f, a)), __fmul_rn(y, a));
}
/* RADIAL (shaders/vkvg_main.frag:109-144): the focus ray from c0 through p
   meets circle 1 at the projection; the gradient runs from r0 to that
   distance (1 where the ray misses).  normalize(v) = v / length(v); dot and
   distance in GLSL's left-to-right order. */
__device__ float    gb_linear_t(const gb_grad &g, float p_x, float p_y);
__device__ uint32_t gb_grad_word(const gb_grad &g, float dist);
__device__ float gb_radial_t(const gb_grad &g, float p_x, float p_y) {
    const float c0x = __fdiv_rn(g.cp[0], g.w), c0y = __fdiv_rn(g.cp[1], g.h);
    const float c1x = __fdiv_rn(g.cp[4], g.w), c1y = __fdiv_rn(g.cp[5], g.h);
    const float r0 = __fdiv_rn(g.cp[2], g.w), r1 = __fdiv_rn(g.cp[6], g.w);
    float       grad_len = 1.0f;
    const float dfx = __fsub_rn(c0x, c1x), dfy = __fsub_rn(c0y, c1y);
    const float vx = __fsub_rn(p_x, c0x), vy = __fsub_rn(p_y, c0y);
    const float len = __fsqrt_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)));
    const float rx = __fdiv_rn(vx, len), ry = __fdiv_rn(vy, len);
    const float a    = __fadd_rn(__fmul_rn(rx, rx), __fmul_rn(ry, ry));
    const float b    = __fmul_rn(2.0f, __fadd_rn(__fmul_rn(rx, dfx), __fmul_rn(ry, dfy)));
    const float cc   = __fsub_rn(__fadd_rn(__fmul_rn(dfx, dfx), __fmul_rn(dfy, dfy)), __fmul_rn(r1, r1));
    const float disc = __fsub_rn(__fmul_rn(b, b), __fmul_rn(__fmul_rn(4.0f, a), cc));
    if (disc >= 0.0f) {
        const float t  = __fdiv_rn(__fadd_rn(-b, __fsqrt_rn(fabsf(disc))), __fmul_rn(2.0f, a));
        const float qx = __fsub_rn(__fadd_rn(c0x, __fmul_rn(rx, t)), c0x);
        const float qy = __fsub_rn(__fadd_rn(c0y, __fmul_rn(ry, t)), c0y);
        grad_len       = __fsub_rn(__fsqrt_rn(__fadd_rn(__fmul_rn(qx, qx), __fmul_rn(qy, qy))), r0);
    }
    return __fdiv_rn(__fsub_rn(len, r0), grad_len);
}
/* SURFACE (shaders/vkvg_main.frag:72-82) through the sampler vkvg builds
   (src/vkvg_context_internal.c:730-755): texel coordinates by the Vulkan
   texel filtering rules, nearest or bilinear with 8-bit weights, the four
   address modes, a transparent black border */
__device__ __forceinline__ int32_t gb_wrap(int32_t i, int32_t n, uint32_t extend) {
    switch (extend) {
    case 1: /* VKVG_EXTEND_REPEAT: VK_SAMPLER_ADDRESS_MODE_REPEAT */
        i %= n;
        return i < 0 ? i + n : i;
    case 2: { /* REFLECT: MIRRORED_REPEAT, (n - 1) - mirror((i mod 2n) - n) */
        int32_t t = i % (2 * n);
        t         = (t < 0 ? t + 2 * n : t) - n;
        return (n - 1) - (t >= 0 ? t : -(1 + t));
    }
    case 3: /* PAD: CLAMP_TO_EDGE */ return min(max(i, 0), n - 1);
    default: /* NONE: CLAMP_TO_BORDER */ return (i < 0 || i >= n) ? -1 : i;
    }
}
/* floor to an integer texel coordinate: NaN gives 0, magnitudes are held
   to 2^30 so that the neighbour i + 1 stays representable */
__device__ __forceinline__ int32_t gb_floor_i(float x) {
    const float f = floorf(x);
    if (!(f == f))
        return 0;
    return (int32_t)fminf(fmaxf(f, -1073741824.0f), 1073741824.0f);
}
__device__ __forceinline__ float4 gb_texel(const gb_grad &g, int32_t i, int32_t j) {
    i = gb_wrap(i, (int32_t)g.sw, g.extend);
    j = gb_wrap(j, (int32_t)g.sh, g.extend);
    if (i < 0 || j < 0)
        return make_float4(0.f, 0.f, 0.f, 0.f);
    const uint32_t t = __ldg(g.texels + (size_t)j * g.sw + i);
    return make_float4(__fdiv_rn((float)(t & 0xFFu), 255.0f), __fdiv_rn((float)((t >> 8) & 0xFFu), 255.0f),
                       __fdiv_rn((float)((t >> 16) & 0xFFu), 255.0f), __fdiv_rn((float)(t >> 24), 255.0f));
}
__device__ uint32_t gb_surface_pixel(const gb_grad &g, uint32_t px, uint32_t py) {
    const float qx = __fsub_rn(__fadd_rn((float)px, 0.5f), g.ox), qy = __fsub_rn(__fadd_rn((float)py, 0.5f), g.oy);
    const float u  = __fdiv_rn(__fadd_rn(__fadd_rn(__fmul_rn(g.m[0], qx), __fmul_rn(g.m[2], qy)), g.m[4]), (float)g.sw);
    const float v  = __fdiv_rn(__fadd_rn(__fadd_rn(__fmul_rn(g.m[1], qx), __fmul_rn(g.m[3], qy)), g.m[5]), (float)g.sh);
    const float us = __fmul_rn(u, (float)g.sw), vs = __fmul_rn(v, (float)g.sh);
    float4      c;
    if (g.filter == 0) {
        c = gb_texel(g, gb_floor_i(us), gb_floor_i(vs));
    } else {
        const float a0 = __fsub_rn(us, 0.5f), b0 = __fsub_rn(vs, 0.5f);
        const float fi = floorf(a0), fj = floorf(b0);
        /* weights quantised to 8 fractional bits */
        const float al = __fmul_rn(floorf(__fmul_rn(__fsub_rn(a0, fi), 256.0f)), 1.0f / 256.0f);
        const float be = __fmul_rn(floorf(__fmul_rn(__fsub_rn(b0, fj), 256.0f)), 1.0f / 256.0f);
        const int32_t i = gb_floor_i(a0), j = gb_floor_i(b0);
        const float4  t00 = gb_texel(g, i, j), t10 = gb_texel(g, i + 1, j);
        const float4  t01 = gb_texel(g, i, j + 1), t11 = gb_texel(g, i + 1, j + 1);
        const float   w00 = __fmul_rn(__fsub_rn(1.0f, al), __fsub_rn(1.0f, be)), w10 = __fmul_rn(al, __fsub_rn(1.0f, be));
        const float   w01 = __fmul_rn(__fsub_rn(1.0f, al), be), w11 = __fmul_rn(al, be);
        auto mixc = [&](float x00, float x10, float x01, float x11) {
            return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w00, x00), __fmul_rn(w10, x10)), __fmul_rn(w01, x01)),
                             __fmul_rn(w11, x11));
        };
        c = make_float4(mixc(t00.x, t10.x, t01.x, t11.x), mixc(t00.y, t10.y, t01.y, t11.y),
                        mixc(t00.z, t10.z, t01.z, t11.z), mixc(t00.w, t10.w, t01.w, t11.w));
    }
    const float cc[4] = {c.x, c.y, c.z, c.w};
    uint32_t    word  = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float x = __fmul_rn(__fmul_rn(cc[k], g.opacity), 255.0f);
        x       = x > 0.0f ? fminf(x, 255.0f) : 0.0f; /* NaN -> 0 */
        word |= (uint32_t)__float2int_rn(x) << (8 * k);
    }
    return word;
}
__device__ uint32_t gb_grad_pixel(const gb_grad &g, uint32_t px, uint32_t py) {
    if (g.type == GB_SRC_SURFACE)
        return gb_surface_pixel(g, px, py);
    const float p_x = __fdiv_rn(__fadd_rn((float)px, 0.5f), g.w), p_y = __fdiv_rn(__fadd_rn((float)py, 0.5f), g.h);
    float       dist;
    if (g.type == GB_GRAD_RADIAL) {
        dist = gb_radial_t(g, p_x, p_y);
    } else {
        dist = gb_linear_t(g, p_x, p_y);
    }
    return gb_grad_word(g, dist);
}
/* LINEAR (shaders/vkvg_main.frag:83-108): signed distance along the axis in
   units of its length */
__device__ float gb_linear_t(const gb_grad &g, float p_x, float p_y) {
    const float p0x = __fdiv_rn(g.cp[0], g.w), p0y = __fdiv_rn(g.cp[1], g.h);
    const float p1x = __fdiv_rn(g.cp[2], g.w), p1y = __fdiv_rn(g.cp[3], g.h);
    const float dx = __fsub_rn(p1x, p0x), dy = __fsub_rn(p1y, p0y);
    const float l  = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    const float ux = __fdiv_rn(dx, l), uy = __fdiv_rn(dy, l);
    float       dist;
    if (uy == 0.0f) {
        const float t = __fdiv_rn(__fsub_rn(p_x, p0x), l);
        dist          = ux < 0.0f ? -t : t;
    } else {
        const float m  = __fdiv_rn(-ux, uy);
        const float bb = __fsub_rn(p0y, __fmul_rn(m, p0x));
        dist = __fdiv_rn(__fdiv_rn(__fsub_rn(__fsub_rn(p_y, __fmul_rn(m, p_x)), bb),
                                   __fsqrt_rn(__fadd_rn(1.0f, __fmul_rn(m, m)))),
                         l);
        if (uy < 0.0f)
            dist = -dist;
    }
    return dist;
}
/* the stop colours at gradient parameter dist, times opacity, to UNORM8 */
__device__ uint32_t gb_grad_word(const gb_grad &g, float dist) {
    float       c[4];
    const float t0 = g_smoothstep(g.stops[0], g.stops[1], dist);
#pragma unroll
    for (int k = 0; k < 4; k++)
        c[k] = g_mix(g.colors[k], g.colors[4 + k], t0);
    for (uint32_t i = 1; i + 1 < g.count; i++) {
        const float t = g_smoothstep(g.stops[i], g.stops[i + 1], dist);
#pragma unroll
        for (int k = 0; k < 4; k++)
            c[k] = g_mix(c[k], g.colors[4 * (i + 1) + k], t);
    }
    uint32_t word = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float v = __fmul_rn(__fmul_rn(c[k], g.opacity), 255.0f);
        v       = v > 0.0f ? fminf(v, 255.0f) : 0.0f; /* NaN -> 0 */
        word |= (uint32_t)__float2int_rn(v) << (8 * k);
    }
    return word;
}
__global__ void gb_gradient_fill(uint32_t W, uint32_t H, const gb_grad *__restrict__ g, uint32_t *__restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)W * H)
        return;
    out[i] = gb_grad_pixel(*g, (uint32_t)(i % W), (uint32_t)(i / W));
}
extern "C" cudaError_t gb_launch_gradient_fill(cudaStream_t st, uint32_t W, uint32_t H, const gb_grad *g,
                                               uint32_t *out) {
    const size_t n = (size_t)W * H;
    if (!n)
        return cudaSuccess;
    gb_gradient_fill<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(W, H, g, out);
    return cudaGetLastError();
}

/* write_to_memory's unpremultiply: one table lookup per colour channel
   (the table holds vkvg's double-precision expression for every (a, p)) */
__global__ void gb_unpremultiply(const uint32_t *__restrict__ in, size_t n, const uint8_t *__restrict__ table,
                                 uint32_t *__restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t v  = in[i];
    const uint32_t a  = v >> 24;
    const uint8_t *ta = table + (a << 8);
    out[i]            = (uint32_t)__ldg(ta + (v & 0xFFu)) | ((uint32_t)__ldg(ta + ((v >> 8) & 0xFFu)) << 8) |
             ((uint32_t)__ldg(ta + ((v >> 16) & 0xFFu)) << 16) | (a << 24);
}
extern "C" cudaError_t gb_launch_unpremultiply(cudaStream_t st, const uint32_t *in, size_t n, const uint8_t *table,
                                               uint32_t *out) {
    if (!n)
        return cudaSuccess;
    gb_unpremultiply<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, n, table, out);
    return cudaGetLastError();
}

template <int NW, bool GRAD>
cudaError_t raster_batch_nw(cudaStream_t st, const gb_raster_args *a, const gb_surf *surfs, const uint4 *items,
                            uint32_t nitems, uint32_t *queue, uint32_t nctas) {
    static std::atomic<bool> configured{false}; /* set once; a second setter is harmless */
    if (!configured.load(std::memory_order_acquire)) {
        cudaError_t e = cudaFuncSetAttribute(gb_raster_batch<NW, GRAD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             XT<NW>::SMEM);
        if (e != cudaSuccess)
            return e;
        configured.store(true, std::memory_order_release);
    }
    gb_raster_batch<NW, GRAD>
        <<<nctas * XT<NW>::MINB, XT<NW>::THREADS, XT<NW>::SMEM, st>>>(*a, surfs, items, nitems, queue);
    return cudaGetLastError();
}
template <bool GRAD>
static cudaError_t raster_batch_form(cudaStream_t st, const gb_raster_args *a, const gb_surf *surfs,
                                     const uint4 *items, uint32_t nitems, uint32_t *queue, uint32_t nctas, int form) {
    if (form == 1)
        return raster_batch_nw<XT_NARROW, GRAD>(st, a, surfs, items, nitems, queue, nctas);
    if (form == 2)
        return raster_batch_nw<XT_MID, GRAD>(st, a, surfs, items, nitems, queue, nctas);
    if (form == 3)
        return raster_batch_nw<XT_TINY, GRAD>(st, a, surfs, items, nitems, queue, nctas);
    if (form == 4)
        return raster_batch_nw<XT_MICRO, GRAD>(st, a, surfs, items, nitems, queue, nctas);
    return raster_batch_nw<XT_WIDE, GRAD>(st, a, surfs, items, nitems, queue, nctas);
}
template <int NW, bool GRAD, bool CLIP> cudaError_t raster_nw(cudaStream_t st, const gb_raster_args *a,
                                                              const gb_clip_args *c) {
    static std::atomic<bool> configured{false}; /* set once; a second setter is harmless */
    if (!configured.load(std::memory_order_acquire)) {
        cudaError_t e = cudaFuncSetAttribute(gb_raster<NW, GRAD, CLIP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             XT<NW>::SMEM);
        if (e != cudaSuccess)
            return e;
        configured.store(true, std::memory_order_release);
    }
    dim3 grid((a->W + XT<NW>::W - 1) / XT<NW>::W, a->nbands);
    gb_raster<NW, GRAD, CLIP><<<grid, XT<NW>::THREADS, XT<NW>::SMEM, st>>>(*a, *c);
    return cudaGetLastError();
}

extern "C" uint32_t gb_raster_tile_width(int form) {
    return form == 1   ? XT<XT_NARROW>::W
           : form == 2 ? XT<XT_MID>::W
           : form == 3 ? XT<XT_TINY>::W
           : form == 4 ? XT<XT_MICRO>::W
                       : XT<XT_WIDE>::W;
}
extern "C" cudaError_t gb_launch_raster_batch(cudaStream_t st, const gb_raster_args *a, const gb_surf *surfs,
                                             const uint4 *items, uint32_t nitems, uint32_t *queue, uint32_t nctas,
                                             int form, int gradients) {
    if (!nitems)
        return cudaSuccess;
    return gradients ? raster_batch_form<true>(st, a, surfs, items, nitems, queue, nctas, form)
                     : raster_batch_form<false>(st, a, surfs, items, nitems, queue, nctas, form);
}
/* frames without gradient draws or clipping run the variants without that
   code; frames with clipping run the wide form */
extern "C" cudaError_t gb_launch_raster(cudaStream_t st, const gb_raster_args *a, const gb_clip_args *c, int gradients,
                                       int clipping, int narrow) {
    if (a->nbands == 0)
        return cudaSuccess;
    if (clipping)
        return gradients ? raster_nw<XT_WIDE, true, true>(st, a, c) : raster_nw<XT_WIDE, false, true>(st, a, c);
    if (narrow == 5)
        return gradients ? raster_nw<XT_MICRO, true, false>(st, a, c) : raster_nw<XT_MICRO, false, false>(st, a, c);
    if (narrow == 2)
        return gradients ? raster_nw<XT_TINY, true, false>(st, a, c) : raster_nw<XT_TINY, false, false>(st, a, c);
    if (narrow)
        return gradients ? raster_nw<XT_NARROW, true, false>(st, a, c) : raster_nw<XT_NARROW, false, false>(st, a, c);
    return gradients ? raster_nw<XT_WIDE, true, false>(st, a, c) : raster_nw<XT_WIDE, false, false>(st, a, c);
}
