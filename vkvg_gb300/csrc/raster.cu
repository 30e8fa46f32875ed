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
 * number of covering triangles.  One thread per primitive of the band walks
 * its edges down the band's sample rows and drops each crossing into a
 * shared-memory counter; a 16-lane suffix scan turns counters into per-sample
 * windings.  The fill rule
 * then decides how many times vkvg's blend is applied: even-odd -> w & 1 (the
 * stencil-INVERT fan of _poly_fill), non-zero -> w != 0 (glutess' NONZERO
 * tessellation), stroke -> w (each overlapping stroke triangle blends once
 * under pipe_OVER).
 *
 * Draws are processed in batches of RB_D: the crossings of all draws of a
 * batch are accumulated into separate counter planes in one phase, then each
 * thread applies the batch's draws to its samples in order.  Stroke triangles
 * lying wholly left or right of the tile are skipped (a closed triangle right
 * of every sample adds +1 and -1 to each row it crosses).
 *
 * Crossing x = x0 + dx*(sy-y0)/dy is found exactly: at the edge's first row an
 * fp32 quotient estimate (error < 0.75 for |q| < 2^22) corrected by one exact
 * 64-bit product test (larger quotients take an exact 64-bit division), then a
 * quotient/remainder walk from row to row.
 *
 * Blend (src/vkvg_device_internal.c:200-209, ONE / ONE_MINUS_SRC_ALPHA on
 * premultiplied UNORM8): d' = s + floor((d*(255-sa) + 127) / 255) per channel,
 * two channels per 32-bit lane, saturating.  At the end the tile writes its
 * samples back and the resolved pixels ((sum + S/2) / S) as 128-bit stores.
 */
#include "gb_types.h"
#include "launch.h"

#include <cuda_runtime.h>

#define RB_D        4               /* draws per batch */
#define CNT_W       (GB_TILE_W + 4) /* counter k (1..256) lives at [k + 3]: 16-byte aligned runs */
#define CNT_PLANE   (GB_BAND_ROWS * CNT_W)
#define RASTER_SMEM (RB_D * CNT_PLANE * 4)

/* ceil(num / den) for den > 0, exact */
__device__ __forceinline__ long long ceil_div_exact(long long num, int32_t den) {
    float qf = __ll2float_rn(num) / (float)den;
    if (fabsf(qf) < 4194304.0f) {
        long long c = (long long)ceilf(qf);
        long long p = c * (long long)den;
        if (p < num)
            c++;
        else if (p - den >= num)
            c--;
        return c;
    }
    long long q = num / den, r = num % den;
    return r > 0 ? q + 1 : q;
}

/* floor(num / den) for den > 0, exact */
__device__ __forceinline__ long long floor_div_exact(long long num, int32_t den) {
    return -ceil_div_exact(-num, den);
}

/* Add one directed edge's crossings of the band's sample rows to the tile's
   counter plane: the exact crossing at the first row, then an exact
   quotient/remainder walk from row to row (rows are `step` apart). */
__device__ __forceinline__ void acc_edge(int32_t x0, int32_t y0, int32_t x1, int32_t y1, int32_t band_r0,
                                         int32_t nrows, uint32_t S, int32_t X0, int32_t TW,
                                         int32_t *__restrict__ plane) {
    if (y0 == y1)
        return;
    const int32_t dir  = y0 < y1 ? 1 : -1;
    const int32_t ylo  = min(y0, y1), yhi = max(y0, y1);
    const int32_t off  = S == 4 ? 32 : 128;
    const int32_t sh   = S == 4 ? 6 : 8; /* row step 64 or 256 units */
    /* rows R with ylo <= off + R*step < yhi: ceil division by a power of two */
    int32_t ra = (int32_t)(((long long)ylo - off + (1 << sh) - 1) >> sh);
    int32_t rb = (int32_t)(((long long)yhi - off + (1 << sh) - 1) >> sh) - 1;
    ra         = max(ra, band_r0);
    rb         = min(rb, min(band_r0 + GB_BAND_ROWS - 1, nrows - 1));
    if (ra > rb)
        return;
    const int32_t tx_lo = X0 * 256 + 32, tx_hi = (X0 + TW - 1) * 256 + 224;
    if (max(x0, x1) < tx_lo)
        return; /* crossings left of every tile sample */
    if (min(x0, x1) > tx_hi) {
        for (int32_t R = ra; R <= rb; R++)
            atomicAdd(&plane[(R - band_r0) * CNT_W + TW + 3], dir);
        return;
    }
    const int32_t   dy  = y1 - y0;
    const int32_t   den = dy < 0 ? -dy : dy;
    const int32_t   dxn = dy < 0 ? x0 - x1 : x1 - x0;
    const int32_t   sy0 = off + (ra << sh);
    const long long num = (long long)dxn * (long long)(sy0 - y0);
    long long       c   = ceil_div_exact(num, den); /* crossing - x0 at row ra, rounded up */
    long long       rem = c * den - num;             /* in [0, den) */
    const long long dl  = (long long)dxn << sh;
    const long long qd  = floor_div_exact(dl, den);
    const long long rd  = dl - qd * den;             /* in [0, den) */
    for (int32_t R = ra; R <= rb; R++) {
        const int32_t ox = S == 4 ? ((R & 3) == 0 ? 96 : (R & 3) == 1 ? 224 : (R & 3) == 2 ? 32 : 160) : 128;
        long long     kt = (((long long)x0 + c - 1 - ox) >> 8) + 1 - X0;
        if (kt > TW)
            kt = TW;
        if (kt > 0)
            atomicAdd(&plane[(R - band_r0) * CNT_W + (int32_t)kt + 3], dir);
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

__global__ void __launch_bounds__(256, 3) gb_raster(gb_raster_args A) {
    extern __shared__ __align__(16) int32_t smem[];

    const uint32_t t = threadIdx.x, r = t >> 4, g = t & 15;
    const uint32_t band    = blockIdx.y;
    const int32_t  X0      = (int32_t)(blockIdx.x * GB_TILE_W);
    const int32_t  TW      = min((int32_t)GB_TILE_W, (int32_t)A.W - X0);
    const int32_t  R       = (int32_t)(band * GB_BAND_ROWS + r);
    const bool     row_ok  = R < (int32_t)A.nrows;
    const int32_t  col0    = (int32_t)(16 * g);
    const int32_t  ncols   = row_ok ? max(0, min(16, TW - col0)) : 0;
    const int32_t  band_r0 = (int32_t)(band * GB_BAND_ROWS);
    const int32_t  tx_lo = X0 * 256 + 32, tx_hi = (X0 + TW - 1) * 256 + 224;
    const uint32_t nd    = A.ndraws;
    const size_t   cb    = (size_t)band * nd;
    const bool     dbg   = A.cov_out != nullptr;
    const uint32_t rpp   = A.S == 4 ? 4 : 1;

    uint32_t  col[16];
    uint32_t *srow = A.samples + (size_t)(row_ok ? R : 0) * A.Wpad + X0 + col0;
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
    for (uint32_t i = t; i < RB_D * CNT_PLANE; i += blockDim.x)
        smem[i] = 0;
    __syncthreads();

    const uint32_t dlo = dbg ? A.cov_draw : A.draw_first;
    const uint32_t dhi = dbg ? A.cov_draw + 1 : nd;
    for (uint32_t d0 = dlo; d0 < dhi; d0 += RB_D) {
        const uint32_t nb = min((uint32_t)RB_D, dhi - d0);
        /* ---- accumulate crossings of the batch */
        bool any = false;
        for (uint32_t j = 0; j < nb; j++) {
            const uint32_t d    = d0 + j;
            const uint32_t kind = A.draws[d].kind;
            if (kind == GB_DRAW_PAINT || kind == GB_DRAW_CLEAR)
                continue;
            const uint32_t lo = A.cell_off[cb + d], hi = A.cell_off[cb + d + 1];
            if (lo == hi)
                continue;
            any            = true;
            int32_t *plane = smem + j * CNT_PLANE;
            if (kind == GB_DRAW_STROKE) {
                for (uint32_t i = lo + t; i < hi; i += blockDim.x) {
                    const uint32_t tr  = A.refs[i];
                    const int4     ta  = A.tri_a[tr], tb = A.tri_b[tr];
                    const int32_t  xmn = min(min(ta.x, ta.z), tb.x), xmx = max(max(ta.x, ta.z), tb.x);
                    if (xmx < tx_lo || xmn > tx_hi)
                        continue; /* wholly left or right: no net coverage in the tile */
                    acc_edge(ta.x, ta.y, ta.z, ta.w, band_r0, (int32_t)A.nrows, A.S, X0, TW, plane);
                    acc_edge(ta.z, ta.w, tb.x, tb.y, band_r0, (int32_t)A.nrows, A.S, X0, TW, plane);
                    acc_edge(tb.x, tb.y, ta.x, ta.y, band_r0, (int32_t)A.nrows, A.S, X0, TW, plane);
                }
            } else {
                for (uint32_t i = lo + t; i < hi; i += blockDim.x) {
                    const int4 ed = A.edges[A.refs[i]];
                    acc_edge(ed.x, ed.y, ed.z, ed.w, band_r0, (int32_t)A.nrows, A.S, X0, TW, plane);
                }
            }
        }
        if (any)
            __syncthreads();
        /* ---- apply the batch's draws in order */
        for (uint32_t j = 0; j < nb; j++) {
            const uint32_t d    = d0 + j;
            const gb_draw &D    = A.draws[d];
            const uint32_t kind = D.kind;
            const uint32_t src = D.src, inv = 255u - (src >> 24), op = D.op;
            if (kind == GB_DRAW_PAINT) {
                if (dbg) {
                    for (int c = 0; c < ncols; c++)
                        A.cov_out[((size_t)(R / rpp) * A.W + X0 + col0 + c) * A.S + R % rpp] = 1;
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
            int4   *cp = reinterpret_cast<int4 *>(smem + j * CNT_PLANE + r * CNT_W + col0 + 4);
            int32_t v[16];
            int32_t L = 0;
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
                        A.cov_out[((size_t)(R / rpp) * A.W + X0 + col0 + c) * A.S + R % rpp] = w;
                    k = 0;
                }
                for (int jj = 0; jj < k; jj++)
                    col[c] = blend(col[c], src, inv, op);
            }
#pragma unroll
            for (int q = 0; q < 4; q++)
                cp[q] = make_int4(0, 0, 0, 0);
        }
        if (any)
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
    /* resolve through shared memory (aliases the counter planes) */
    __syncthreads();
    uint32_t *stage = reinterpret_cast<uint32_t *>(smem);
#pragma unroll
    for (int c = 0; c < 16; c++)
        stage[r * GB_TILE_W + col0 + c] = col[c];
    __syncthreads();
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
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(gb_raster, cudaFuncAttributeMaxDynamicSharedMemorySize, RASTER_SMEM);
        if (e != cudaSuccess)
            return e;
        configured = true;
    }
    if (a->nbands == 0)
        return cudaSuccess;
    dim3 grid((a->W + GB_TILE_W - 1) / GB_TILE_W, a->nbands);
    gb_raster<<<grid, 256, RASTER_SMEM, st>>>(*a);
    return cudaGetLastError();
}
