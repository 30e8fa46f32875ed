/*
 * K5 - per-band coverage and compositing on sm_103a.
 *
 * One CTA owns a tile of 256 pixels x 16 sample rows (4 pixel rows at 4x
 * MSAA) and walks the frame's draws in submission order.  Thread (r, g) owns
 * 16 consecutive samples of sample row r; their premultiplied RGBA8 values
 * stay in registers for the whole frame.
 *
 * Coverage is exact integer arithmetic on the snapped 24.8 vertices: an edge
 * crossing sample row y at x_c adds its direction (+1 downward, -1 upward) to
 * every sample with x < x_c (a sample on the edge counts as if moved by
 * (+e, +e^2), which is the top-left rule).  Summed over a closed polygon this
 * is its winding number; summed over positively oriented triangles it is the
 * number of covering triangles.  Each edge touching the band drops its
 * crossings into shared-memory counters (one exact division per edge, then an
 * incremental remainder walk down the rows), and a 16-lane suffix scan turns
 * counters into per-sample windings.  The fill rule then decides how many
 * times vkvg's blend is applied: even-odd -> w & 1 (the stencil-INVERT fan of
 * _poly_fill), non-zero -> w != 0 (glutess' NONZERO tessellation), stroke -> w
 * (each overlapping stroke triangle blends once under pipe_OVER).
 *
 * Blend (src/vkvg_device_internal.c:200-209, ONE / ONE_MINUS_SRC_ALPHA on
 * premultiplied UNORM8): d' = s + floor((d*(255-sa) + 127) / 255) per channel,
 * two channels per 32-bit lane, saturating.  At the end the tile writes its
 * samples back and the resolved pixels ((sum + S/2) / S) as 128-bit stores.
 */
#include "gb_types.h"
#include "launch.h"

#include <cuda_runtime.h>



#define CNT_PAD 4 /* counter k (1..256) lives at [r][k + 3]: 16-byte aligned runs */

__device__ __forceinline__ long long floordiv_ll(long long a, long long b) {
    long long q = a / b;
    if ((a % b != 0) && (a < 0))
        q--;
    return q;
}

/* accumulate one directed edge's crossings of the tile's sample rows */
__device__ __forceinline__ void acc_edge(int32_t x0, int32_t y0, int32_t x1, int32_t y1, int32_t band_r0,
                                         int32_t nrows, uint32_t S, int32_t X0, int32_t TW,
                                         int32_t (*cnt)[GB_TILE_W + CNT_PAD]) {
    if (y0 == y1)
        return;
    int32_t   dir  = y0 < y1 ? 1 : -1;
    int32_t   ylo  = min(y0, y1), yhi = max(y0, y1);
    long long off  = S == 4 ? 32 : 128;
    long long step = S == 4 ? 64 : 256;
    /* rows with ylo <= sy < yhi */
    long long a  = (long long)ylo - off, b = (long long)yhi - off;
    long long ra = -floordiv_ll(-a, step);
    long long rb = -floordiv_ll(-b, step) - 1;
    long long lo = band_r0, hi = min(band_r0 + GB_BAND_ROWS - 1, nrows - 1);
    if (ra < lo)
        ra = lo;
    if (rb > hi)
        rb = hi;
    if (ra > rb)
        return;
    int32_t   xmin = min(x0, x1), xmax = max(x0, x1);
    long long tx_lo = (long long)X0 * 256 + 32, tx_hi = (long long)(X0 + TW - 1) * 256 + 224;
    if ((long long)xmax < tx_lo)
        return; /* crossings left of every tile sample */
    if ((long long)xmin > tx_hi) {
        for (long long R = ra; R <= rb; R++)
            atomicAdd(&cnt[R - band_r0][TW + 3], dir);
        return;
    }
    long long dx = (long long)x1 - x0, dy = (long long)y1 - y0;
    long long den = dy < 0 ? -dy : dy;
    long long dxn = dy < 0 ? -dx : dx;
    long long sy0 = off + step * ra;
    long long num = dxn * (sy0 - y0);
    long long c   = -floordiv_ll(-num, den); /* ceil(num/den) */
    long long rem = c * den - num;
    long long dl  = dxn * step;
    long long qd  = floordiv_ll(dl, den);
    long long rd  = dl - qd * den;
    for (long long R = ra; R <= rb; R++) {
        long long ox = S == 4 ? ((R & 3) == 0 ? 96 : (R & 3) == 1 ? 224 : (R & 3) == 2 ? 32 : 160) : 128;
        long long M  = (long long)x0 + c - 1;
        long long kg = ((M - ox) >> 8) + 1;
        long long kt = kg - X0;
        if (kt > TW)
            kt = TW;
        if (kt > 0)
            atomicAdd(&cnt[R - band_r0][kt + 3], dir);
        rem -= rd;
        c += qd;
        if (rem < 0) {
            rem += den;
            c += 1;
        }
    }
}

__device__ __forceinline__ uint32_t div255_2x(uint32_t x) {
    /* per 16-bit lane: floor(x / 255) for x <= 65152 */
    return ((x + ((x >> 8) & 0x00FF00FFu) + 0x00010001u) >> 8) & 0x00FF00FFu;
}
/* t = floor((d * inv + 127) / 255) per channel */
__device__ __forceinline__ uint32_t scaled_dst(uint32_t d, uint32_t inv) {
    uint32_t rb = (d & 0x00FF00FFu) * inv + 0x007F007Fu;
    uint32_t ag = ((d >> 8) & 0x00FF00FFu) * inv + 0x007F007Fu;
    return div255_2x(rb) | (div255_2x(ag) << 8);
}
__device__ __forceinline__ uint32_t blend(uint32_t d, uint32_t s, uint32_t inv, uint32_t op) {
    if (op == GB_OP_CLEAR)
        return 0u;
    uint32_t t = scaled_dst(d, inv);
    if (op == GB_OP_DIFFERENCE)
        return __vsubus4(s, t);
    return __vaddus4(s, t);
}

__global__ void __launch_bounds__(256) gb_raster(gb_raster_args A) {
    __shared__ __align__(16) int32_t  cnt[GB_BAND_ROWS][GB_TILE_W + CNT_PAD];
    __shared__ __align__(16) uint32_t stage[GB_BAND_ROWS * GB_TILE_W];

    const uint32_t t = threadIdx.x, r = t >> 4, g = t & 15;
    const uint32_t band = blockIdx.y;
    const int32_t  X0   = (int32_t)(blockIdx.x * GB_TILE_W);
    const int32_t  TW   = min((int32_t)GB_TILE_W, (int32_t)A.W - X0);
    const int32_t  R    = (int32_t)(band * GB_BAND_ROWS + r);
    const bool     row_ok = R < (int32_t)A.nrows;
    const int32_t  col0   = (int32_t)(16 * g);
    const int32_t  ncols  = row_ok ? max(0, min(16, TW - col0)) : 0;
    const int32_t  band_r0 = (int32_t)(band * GB_BAND_ROWS);

    /* skip bands no draw touches (unless a paint / clear covers everything) */
    const uint32_t nd  = A.ndraws;
    const size_t   cb  = (size_t)band * nd;

    uint32_t col[16];
    uint32_t *srow = A.samples + (size_t)(R < (int32_t)A.nrows ? R : 0) * A.Wpad + X0 + col0;
    if (A.init_mode == 1) {
#pragma unroll
        for (int c = 0; c < 16; c++)
            col[c] = A.init_color;
    } else if (ncols == 16) {
        const uint4 *p = reinterpret_cast<const uint4 *>(srow);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            uint4 v        = p[q];
            col[4 * q]     = v.x;
            col[4 * q + 1] = v.y;
            col[4 * q + 2] = v.z;
            col[4 * q + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int c = 0; c < 16; c++)
            col[c] = c < ncols ? srow[c] : 0u;
    }
    for (uint32_t i = t; i < GB_BAND_ROWS * (GB_TILE_W + CNT_PAD); i += blockDim.x)
        (&cnt[0][0])[i] = 0;
    __syncthreads();

    const bool     dbg   = A.cov_out != nullptr;
    const uint32_t dlo   = dbg ? A.cov_draw : A.draw_first;
    const uint32_t dhi   = dbg ? A.cov_draw + 1 : nd;
    const uint32_t rppx  = A.S == 4 ? 4 : 1;
    for (uint32_t d = dlo; d < dhi; d++) {
        const gb_draw &D    = A.draws[d];
        const uint32_t kind = D.kind;
        const uint32_t src = D.src, inv = 255u - (src >> 24), op = D.op;
        if (kind == GB_DRAW_PAINT) {
            if (dbg) {
                for (int c = 0; c < ncols; c++)
                    A.cov_out[((size_t)(R / rppx) * A.W + X0 + col0 + c) * A.S + R % rppx] = 1;
                continue;
            }
#pragma unroll
            for (int c = 0; c < 16; c++)
                col[c] = blend(col[c], src, inv, op);
            continue;
        }
        if (kind == GB_DRAW_CLEAR) {
#pragma unroll
            for (int c = 0; c < 16; c++)
                col[c] = 0u;
            continue;
        }
        const uint32_t lo = A.cell_off[cb + d], hi = A.cell_off[cb + d + 1];
        if (lo == hi)
            continue;
        if (kind == GB_DRAW_STROKE) {
            for (uint32_t i = lo + t; i < hi; i += blockDim.x) {
                uint32_t tr = A.refs[i];
                int4     ta = A.tri_a[tr], tb = A.tri_b[tr];
                acc_edge(ta.x, ta.y, ta.z, ta.w, band_r0, (int32_t)A.nrows, A.S, X0, TW, cnt);
                acc_edge(ta.z, ta.w, tb.x, tb.y, band_r0, (int32_t)A.nrows, A.S, X0, TW, cnt);
                acc_edge(tb.x, tb.y, ta.x, ta.y, band_r0, (int32_t)A.nrows, A.S, X0, TW, cnt);
            }
        } else {
            for (uint32_t i = lo + t; i < hi; i += blockDim.x) {
                int4 e = A.edges[A.refs[i]];
                acc_edge(e.x, e.y, e.z, e.w, band_r0, (int32_t)A.nrows, A.S, X0, TW, cnt);
            }
        }
        __syncthreads();
        /* counters k = col0+1 .. col0+16 */
        int32_t   v[16];
        int4     *cp = reinterpret_cast<int4 *>(&cnt[r][col0 + 4]);
        int32_t   L  = 0;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            int4 x       = cp[q];
            v[4 * q]     = x.x;
            v[4 * q + 1] = x.y;
            v[4 * q + 2] = x.z;
            v[4 * q + 3] = x.w;
            L += x.x + x.y + x.z + x.w;
        }
        int32_t incl = L;
#pragma unroll
        for (int o = 1; o < 16; o <<= 1) {
            int32_t u = __shfl_down_sync(0xffffffffu, incl, o, 16);
            if (g + o < 16)
                incl += u;
        }
        int32_t w = incl - L;
#pragma unroll
        for (int c = 15; c >= 0; c--) {
            w += v[c];
            int32_t k;
            if (kind == GB_DRAW_FILL_EO)
                k = w & 1;
            else if (kind == GB_DRAW_FILL_NZ)
                k = w != 0;
            else
                k = w > 0 ? w : 0;
            if (c >= ncols)
                k = 0;
            if (dbg) {
                if (c < ncols)
                    A.cov_out[((size_t)(R / rppx) * A.W + X0 + col0 + c) * A.S + R % rppx] = w;
                k = 0;
            }
            for (int j = 0; j < k; j++)
                col[c] = blend(col[c], src, inv, op);
        }
#pragma unroll
        for (int q = 0; q < 4; q++)
            cp[q] = make_int4(0, 0, 0, 0);
        __syncthreads();
    }
    if (dbg)
        return;

    /* write back samples */
    if (ncols == 16) {
        uint4 *p = reinterpret_cast<uint4 *>(srow);
#pragma unroll
        for (int q = 0; q < 4; q++)
            p[q] = make_uint4(col[4 * q], col[4 * q + 1], col[4 * q + 2], col[4 * q + 3]);
    } else {
#pragma unroll
        for (int c = 0; c < 16; c++)
            if (c < ncols)
                srow[c] = col[c];
    }
    /* resolve */
#pragma unroll
    for (int c = 0; c < 16; c++)
        stage[r * GB_TILE_W + col0 + c] = col[c];
    __syncthreads();
    const uint32_t rpp   = A.S == 4 ? 4 : 1;
    const uint32_t prows = GB_BAND_ROWS / rpp;
    const uint32_t npx   = prows * GB_TILE_W;
    for (uint32_t q = t * 4; q < npx; q += blockDim.x * 4) {
        uint32_t pr = q / GB_TILE_W, px = q % GB_TILE_W; /* 4 consecutive pixels px..px+3 */
        uint32_t py = band * prows + pr;
        if (py >= A.H || (int32_t)px >= TW)
            continue;
        uint32_t outp[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            uint32_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
            for (uint32_t s = 0; s < rpp; s++) {
                uint32_t v = stage[(pr * rpp + s) * GB_TILE_W + px + k];
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

extern "C" cudaError_t gb_launch_raster(cudaStream_t st, const gb_raster_args *a) {
    if (a->nbands == 0)
        return cudaSuccess;
    dim3 grid((a->W + GB_TILE_W - 1) / GB_TILE_W, a->nbands);
    gb_raster<<<grid, 256, 0, st>>>(*a);
    return cudaGetLastError();
}
