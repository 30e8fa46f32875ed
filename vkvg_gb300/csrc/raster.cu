/*
 * K5 - per-band coverage and compositing on sm_103a.
 *
 * One CTA (16 warps) owns a tile of up to 1024 pixels x 16 sample rows (4
 * pixel rows at 4x MSAA) and walks the frame's draws in submission order.
 * Warp r owns sample row r; lane l owns its 32 consecutive samples, whose
 * premultiplied RGBA8 values stay in registers for the whole frame.
 *
 * Coverage is exact integer arithmetic.  The crossing kernels (setup.cu)
 * record, for every edge and every sample row it crosses, k = the number of
 * that row's samples lying left of the crossing, and the edge's direction.
 * An edge adds its direction to every sample left of its crossing (a sample
 * on the edge counts as if moved by (+e, +e^2): the top-left rule), so the
 * suffix sum of the records over a row is the winding number for a closed
 * polygon, or the covering-triangle count for positively oriented triangles.
 * Per draw, the CTA drops the draw's records of its band into shared-memory
 * counters, each warp suffix-scans its row with shuffles, and the fill rule
 * decides how many times vkvg's blend is applied per sample: even-odd ->
 * w & 1 (the stencil-INVERT fan of _poly_fill), non-zero -> w != 0 (glutess'
 * NONZERO tessellation), stroke -> w (each overlapping stroke triangle blends
 * once under pipe_OVER).  Lanes whose counters no record touched take a
 * uniform-winding fast path.  XT_D draws share one pair of barriers.
 *
 * Blend (src/vkvg_device_internal.c:200-209, ONE / ONE_MINUS_SRC_ALPHA on
 * premultiplied UNORM8): d' = s + floor((d*(255-sa) + 127) / 255) per channel,
 * two channels per 32-bit lane, saturating.  At the end the tile writes its
 * samples back and the resolved pixels ((sum + S/2) / S) as 128-bit stores.
 */
#include "gb_types.h"
#include "launch.h"

#include <cuda_runtime.h>

#define XT_W        1024                 /* tile width in pixels */
#define XT_THREADS  512                  /* 16 warps: one per sample row */
#define XT_D        2                    /* draws per barrier pair */
#define XCNT_W      (XT_W + 4)           /* counter k (1..1024) at [k + 3]: 16-byte aligned lane runs */
#define XPLANE      (GB_BAND_ROWS * XCNT_W + GB_BAND_ROWS) /* counters + one touched mask per row */
#define RASTER_SMEM (XT_D * XPLANE * 4)

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
__device__ __forceinline__ int32_t rule(uint32_t kind, int32_t w) {
    if (kind == GB_DRAW_FILL_EO)
        return w & 1;
    if (kind == GB_DRAW_FILL_NZ)
        return w != 0;
    return w > 0 ? w : 0;
}

__global__ void __launch_bounds__(XT_THREADS, 1) gb_raster(gb_raster_args A) {
    extern __shared__ __align__(16) int32_t smem[];

    const uint32_t t = threadIdx.x, r = t >> 5, l = t & 31;
    const uint32_t band    = blockIdx.y;
    const int32_t  X0      = (int32_t)(blockIdx.x * XT_W);
    const int32_t  TW      = min((int32_t)XT_W, (int32_t)A.W - X0);
    const int32_t  R       = (int32_t)(band * GB_BAND_ROWS + r);
    const bool     row_ok  = R < (int32_t)A.nrows;
    const int32_t  col0    = (int32_t)(32 * l);
    const int32_t  ncols   = row_ok ? max(0, min(32, TW - col0)) : 0;
    const uint32_t nd      = A.ndraws;
    const size_t   cb      = (size_t)band * nd;
    const bool     dbg     = A.cov_out != nullptr;
    const uint32_t rpp     = A.S == 4 ? 4 : 1;

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
    for (uint32_t i = t; i < XT_D * XPLANE; i += XT_THREADS)
        smem[i] = 0;
    __syncthreads();

    const uint32_t dlo = dbg ? A.cov_draw : A.draw_first;
    const uint32_t dhi = dbg ? A.cov_draw + 1 : nd;
    for (uint32_t d0 = dlo; d0 < dhi; d0 += XT_D) {
        const uint32_t nb = min((uint32_t)XT_D, dhi - d0);
        /* ---- drop the batch's crossing records into the counters */
        bool any = false;
        for (uint32_t j = 0; j < nb; j++) {
            const uint32_t d  = d0 + j;
            const uint32_t lo = A.cell_off[cb + d], hi = A.cell_off[cb + d + 1];
            if (lo == hi)
                continue;
            any             = true;
            int32_t  *plane = smem + j * XPLANE;
            uint32_t *touch = reinterpret_cast<uint32_t *>(plane + GB_BAND_ROWS * XCNT_W);
            for (uint32_t i = lo + t; i < hi; i += XT_THREADS) {
                const uint32_t rec = A.xings[i];
                int32_t        k   = (int32_t)(rec >> 5) - X0;
                if (k <= 0)
                    continue; /* no sample of this tile lies left of the crossing */
                if (k > TW)
                    k = TW;
                const uint32_t rr = rec & (GB_BAND_ROWS - 1);
                atomicAdd(&plane[rr * XCNT_W + k + 3], (rec & 16u) ? 1 : -1);
                atomicOr(&touch[rr], 1u << ((k - 1) >> 5));
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
                for (int c = 0; c < 32; c++)
                    col[c] = blend(col[c], src, inv, op);
                continue;
            }
            if (kind == GB_DRAW_CLEAR) {
#pragma unroll
                for (int c = 0; c < 32; c++)
                    col[c] = 0u;
                continue;
            }
            const uint32_t lo = A.cell_off[cb + d], hi = A.cell_off[cb + d + 1];
            if (lo == hi)
                continue;
            int32_t       *plane = smem + j * XPLANE;
            uint32_t      *touch = reinterpret_cast<uint32_t *>(plane + GB_BAND_ROWS * XCNT_W);
            const uint32_t tm    = touch[r];
            const bool     mine  = (tm >> l) & 1u;
            int4          *cp    = reinterpret_cast<int4 *>(plane + r * XCNT_W + col0 + 4);
            int32_t        L     = 0;
            if (mine) {
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    int4 x = cp[q];
                    L += x.x + x.y + x.z + x.w;
                }
            }
            int32_t incl = L;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int32_t u = __shfl_down_sync(0xffffffffu, incl, o);
                if (l + o < 32)
                    incl += u;
            }
            const int32_t E = incl - L; /* records right of this lane's samples */
            if (dbg) {
                int32_t w = E;
                for (int c = 31; c >= 0; c--) {
                    if (mine)
                        w += plane[r * XCNT_W + col0 + c + 4];
                    if (c < ncols)
                        A.cov_out[((size_t)(R / rpp) * A.W + X0 + col0 + c) * A.S + R % rpp] = w;
                }
            } else if (!mine) {
                const int32_t k = ncols ? rule(kind, E) : 0;
                for (int jj = 0; jj < k; jj++) {
#pragma unroll
                    for (int c = 0; c < 32; c++)
                        col[c] = blend(col[c], src, inv, op);
                }
            } else {
                int32_t w = E;
#pragma unroll
                for (int q = 7; q >= 0; q--) {
                    int4 x = cp[q];
#pragma unroll
                    for (int e = 3; e >= 0; e--) {
                        const int c = 4 * q + e;
                        w += e == 3 ? x.w : e == 2 ? x.z : e == 1 ? x.y : x.x;
                        int32_t k = c < ncols ? rule(kind, w) : 0;
                        for (int jj = 0; jj < k; jj++)
                            col[c] = blend(col[c], src, inv, op);
                    }
                }
            }
            if (mine) {
#pragma unroll
                for (int q = 0; q < 8; q++)
                    cp[q] = make_int4(0, 0, 0, 0);
            }
            __syncwarp();
            if (l == 0)
                touch[r] = 0u;
        }
        if (any)
            __syncthreads();
    }
    if (dbg)
        return;

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
    /* resolve through shared memory (aliases the counter planes) */
    __syncthreads();
    uint32_t *stage = reinterpret_cast<uint32_t *>(smem);
#pragma unroll
    for (int c = 0; c < 32; c++)
        stage[r * XT_W + col0 + c] = col[c];
    __syncthreads();
    const uint32_t prows = GB_BAND_ROWS / rpp;
    const uint32_t npx   = prows * XT_W;
    for (uint32_t q = t * 4; q < npx; q += XT_THREADS * 4) {
        uint32_t pr = q / XT_W, px = q % XT_W; /* 4 consecutive pixels px..px+3 */
        uint32_t py = band * prows + pr;
        if (py >= A.H || (int32_t)px >= TW)
            continue;
        uint32_t outp[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            uint32_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
            for (uint32_t s = 0; s < rpp; s++) {
                uint32_t v = stage[(pr * rpp + s) * XT_W + px + k];
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
    dim3 grid((a->W + XT_W - 1) / XT_W, a->nbands);
    gb_raster<<<grid, XT_THREADS, RASTER_SMEM, st>>>(*a);
    return cudaGetLastError();
}
