/*
 * K7/K8 (flattening part) - the analytic-coverage mode's flattening and its
 * adjoint, sm_103a.
 *
 * One warp per segment.  A segment starts at its first control point and
 * ends at the next segment's start (the contour's first for the last one);
 * it adds its start point, then, for a cubic, the interior points of vkvg's
 * _recursive_bezier walk (src/vkvg_context_internal.c:1313-1461) at vkvg's
 * default tolerance 0.25 (src/vkvg_context.c:558).  Concatenated, the
 * segments of a contour give exactly the points vkvg's move_to / curve_to /
 * close_path sequence leaves in its path.
 *
 * Cubics are walked breadth first by the warp (gb_bezier_warp), or serially
 * by one lane when the tree outgrows the warp's buffers; both give vkvg's
 * points in vkvg's order.  Scenes of small curves (a few points per
 * segment on average) take one lane per segment instead, each walking its
 * cubic serially.
 *
 * The backward pass walks the same subdivision again instead of storing it:
 * every emitted point is the blossom of its sub-curve interval, a fixed
 * linear combination of the four control points (gb_bez_weights), so
 * dL/dcontrol = sum over the segment's points of weight * dL/dpoint.
 *
 * Built with -fmad=false and IEEE division (geometry unit), so the decisions
 * and the points are those of the plain flatten kernels and of the oracle.
 */
#include "analytic.h"
#include "bezier.cuh"

#include <cuda_runtime.h>

#define AK_TOL 0.25f

__device__ __forceinline__ bool ak_fin(float v) { return (__float_as_uint(v) & 0x7f800000u) != 0x7f800000u; }

struct ak_cnt_emit {
    uint32_t n;
    __device__ void operator()(float x, float y, int, float, float) {
        if (!(x != x || y != y))
            n++;
    }
};
/* a point's neighbours in its closed contour [c0, c1) */
__device__ __forceinline__ uint2 ak_nb(uint32_t o, uint32_t c0, uint32_t c1) {
    return make_uint2(o == c0 ? c1 - 1 : o - 1, o + 1 == c1 ? c0 : o + 1);
}
struct ak_pt_emit {
    float2   *pts;
    uint2    *nb;
    uint32_t  o, c0, c1;
    __device__ void operator()(float x, float y, int, float, float) {
        if (x != x || y != y)
            return;
        pts[o] = make_float2(x, y);
        nb[o]  = ak_nb(o, c0, c1);
        o++;
    }
};
struct ak_grad_emit {
    const float2 *g;
    uint32_t      o;
    float2        gc[4];
    __device__ void operator()(float x, float y, int which, float ta, float tb) {
        if (x != x || y != y)
            return;
        float  w[4];
        float2 d = g[o++];
        gb_bez_weights(which, ta, tb, w);
#pragma unroll
        for (int k = 0; k < 4; k++)
            gc[k].x += w[k] * d.x, gc[k].y += w[k] * d.y;
    }
};

__device__ __forceinline__ bool ak_cubic_cp(const ak_scene &S, const float2 *ctrl, uint32_t s, float2 c[4]) {
    uint32_t c0 = S.seg_cp[s];
    c[0] = ctrl[c0], c[1] = ctrl[c0 + 1], c[2] = ctrl[c0 + 2], c[3] = ctrl[S.seg_end[s]];
    bool fin = true;
#pragma unroll
    for (int k = 0; k < 4; k++)
        fin = fin && ak_fin(c[k].x) && ak_fin(c[k].y);
    return fin;
}

/* One warp per segment: the breadth-first walk of bezier.cuh, or, for a tree
   it cannot hold, the serial walk on lane 0.  The start point comes first. */
#define AK_FW 4 /* warps per block */

__device__ __forceinline__ bool seg_start(const ak_scene &S, const float2 *ctrl, uint32_t s, float2 &p) {
    p = ctrl[S.seg_cp[s]];
    return !(p.x != p.x || p.y != p.y);
}

__global__ void __launch_bounds__(32 * AK_FW) ak_flat_count(ak_scene S, const float2 *__restrict__ ctrl,
                                                           uint32_t *__restrict__ cnt) {
    __shared__ gb_bw_smem sm[AK_FW];
    uint32_t              w = threadIdx.x >> 5, lane = threadIdx.x & 31, s = blockIdx.x * AK_FW + w;
    if (s >= S.nseg)
        return;
    float2   p, c[4];
    uint32_t n = seg_start(S, ctrl, s, p) ? 1u : 0u;
    if (S.seg_kind[s] == AK_SEG_CUBIC && ak_cubic_cp(S, ctrl, s, c)) {
        int m = gb_bezier_warp(AK_TOL, c[0].x, c[0].y, c[1].x, c[1].y, c[2].x, c[2].y, c[3].x, c[3].y, sm[w]);
        if (m < 0) {
            ak_cnt_emit e{0};
            if (lane == 0)
                gb_bezier_walk<false>(AK_TOL, c[0].x, c[0].y, c[1].x, c[1].y, c[2].x, c[2].y, c[3].x, c[3].y, e);
            m = (int)e.n;
        }
        n += (uint32_t)m;
    }
    if (lane == 0)
        cnt[s] = n;
}

__global__ void __launch_bounds__(32 * AK_FW) ak_flat_emit(ak_scene S, const float2 *__restrict__ ctrl,
                                                          const uint32_t *__restrict__ off, float2 *__restrict__ pts,
                                                          uint2 *__restrict__ pt_nb, uint32_t cap,
                                                          uint32_t *__restrict__ status) {
    __shared__ gb_bw_smem sm[AK_FW];
    uint32_t              w = threadIdx.x >> 5, lane = threadIdx.x & 31, s = blockIdx.x * AK_FW + w;
    if (off[S.nseg] > cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            atomicOr(status, AK_ERR_POINTS);
        return;
    }
    if (s >= S.nseg)
        return;
    float2         p, c[4];
    const uint32_t cont = S.seg_contour[s];
    const uint32_t c0 = off[S.cont_s0[cont]], c1 = off[S.cont_s0[cont + 1]];
    uint32_t       o  = off[s];
    if (seg_start(S, ctrl, s, p)) {
        if (lane == 0)
            pts[o] = p, pt_nb[o] = ak_nb(o, c0, c1);
        o++;
    }
    if (S.seg_kind[s] == AK_SEG_CUBIC && ak_cubic_cp(S, ctrl, s, c)) {
        int m = gb_bezier_warp(AK_TOL, c[0].x, c[0].y, c[1].x, c[1].y, c[2].x, c[2].y, c[3].x, c[3].y, sm[w]);
        if (m < 0) {
            if (lane == 0) {
                ak_pt_emit e{pts, pt_nb, o, c0, c1};
                gb_bezier_walk<false>(AK_TOL, c[0].x, c[0].y, c[1].x, c[1].y, c[2].x, c[2].y, c[3].x, c[3].y, e);
            }
            return;
        }
        for (int i = (int)lane; i < m; i += 32) {
            int r        = gb_bw_rank(sm[w], m, i);
            pts[o + r]   = sm[w].pt[i].p;
            pt_nb[o + r] = ak_nb(o + r, c0, c1);
        }
    }
}

__global__ void __launch_bounds__(32 * AK_FW) ak_flat_bwd(ak_scene S, const float2 *__restrict__ ctrl,
                                                         const uint32_t *__restrict__ off, uint32_t cap,
                                                         const float2 *__restrict__ gpts,
                                                         float2 *__restrict__ gctrl) {
    __shared__ gb_bw_smem sm[AK_FW];
    uint32_t              w = threadIdx.x >> 5, lane = threadIdx.x & 31, s = blockIdx.x * AK_FW + w;
    if (s >= S.nseg || off[S.nseg] > cap)
        return;
    uint32_t c0 = S.seg_cp[s], o = off[s];
    float2   p, c[4], gc[4];
#pragma unroll
    for (int k = 0; k < 4; k++)
        gc[k] = make_float2(0.f, 0.f);
    if (seg_start(S, ctrl, s, p)) {
        if (lane == 0)
            gc[0] = gpts[o];
        o++;
    }
    bool cubic = S.seg_kind[s] == AK_SEG_CUBIC;
    if (cubic && ak_cubic_cp(S, ctrl, s, c)) {
        int m = gb_bezier_warp(AK_TOL, c[0].x, c[0].y, c[1].x, c[1].y, c[2].x, c[2].y, c[3].x, c[3].y, sm[w]);
        if (m < 0) {
            if (lane == 0) {
                ak_grad_emit e;
                e.g = gpts, e.o = o;
#pragma unroll
                for (int k = 0; k < 4; k++)
                    e.gc[k] = gc[k];
                gb_bezier_walk<true>(AK_TOL, c[0].x, c[0].y, c[1].x, c[1].y, c[2].x, c[2].y, c[3].x, c[3].y, e);
#pragma unroll
                for (int k = 0; k < 4; k++)
                    gc[k] = e.gc[k];
            }
        } else {
            for (int i = (int)lane; i < m; i += 32) {
                float2 d  = gpts[o + gb_bw_rank(sm[w], m, i)];
                float2 ti = gb_bw_interval(sm[w].pt[i]);
                float  wt[4];
                gb_bez_weights(sm[w].pt[i].which, ti.x, ti.y, wt);
#pragma unroll
                for (int k = 0; k < 4; k++)
                    gc[k].x += wt[k] * d.x, gc[k].y += wt[k] * d.y;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++)
        for (int q = 16; q > 0; q >>= 1) {
            gc[k].x += __shfl_xor_sync(0xffffffffu, gc[k].x, q);
            gc[k].y += __shfl_xor_sync(0xffffffffu, gc[k].y, q);
        }
    if (lane == 0) {
        atomicAdd(&gctrl[c0].x, gc[0].x), atomicAdd(&gctrl[c0].y, gc[0].y);
        if (cubic) {
            atomicAdd(&gctrl[c0 + 1].x, gc[1].x), atomicAdd(&gctrl[c0 + 1].y, gc[1].y);
            atomicAdd(&gctrl[c0 + 2].x, gc[2].x), atomicAdd(&gctrl[c0 + 2].y, gc[2].y);
            uint32_t ce = S.seg_end[s];
            atomicAdd(&gctrl[ce].x, gc[3].x), atomicAdd(&gctrl[ce].y, gc[3].y);
        }
    }
}

/* One lane per segment, each walking its cubic serially: for scenes of
   small curves (a few points each), where a warp per segment would leave
   most lanes idle.  The same points in the same order. */
#define AK_LT 256 /* lanes per block */

__global__ void __launch_bounds__(AK_LT) ak_flat_count_lane(ak_scene S, const float2 *__restrict__ ctrl,
                                                           uint32_t *__restrict__ cnt) {
    const uint32_t s = blockIdx.x * AK_LT + threadIdx.x;
    if (s >= S.nseg)
        return;
    float2   p, c[4];
    uint32_t n = seg_start(S, ctrl, s, p) ? 1u : 0u;
    if (S.seg_kind[s] == AK_SEG_CUBIC && ak_cubic_cp(S, ctrl, s, c)) {
        ak_cnt_emit e{0};
        gb_bezier_walk<false>(AK_TOL, c[0].x, c[0].y, c[1].x, c[1].y, c[2].x, c[2].y, c[3].x, c[3].y, e);
        n += e.n;
    }
    cnt[s] = n;
}

__global__ void __launch_bounds__(AK_LT) ak_flat_emit_lane(ak_scene S, const float2 *__restrict__ ctrl,
                                                          const uint32_t *__restrict__ off, float2 *__restrict__ pts,
                                                          uint2 *__restrict__ pt_nb, uint32_t cap,
                                                          uint32_t *__restrict__ status) {
    const uint32_t s = blockIdx.x * AK_LT + threadIdx.x;
    if (off[S.nseg] > cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            atomicOr(status, AK_ERR_POINTS);
        return;
    }
    if (s >= S.nseg)
        return;
    float2         p, c[4];
    const uint32_t cont = S.seg_contour[s];
    const uint32_t c0 = off[S.cont_s0[cont]], c1 = off[S.cont_s0[cont + 1]];
    uint32_t       o  = off[s];
    if (seg_start(S, ctrl, s, p)) {
        pts[o] = p, pt_nb[o] = ak_nb(o, c0, c1);
        o++;
    }
    if (S.seg_kind[s] == AK_SEG_CUBIC && ak_cubic_cp(S, ctrl, s, c)) {
        ak_pt_emit e{pts, pt_nb, o, c0, c1};
        gb_bezier_walk<false>(AK_TOL, c[0].x, c[0].y, c[1].x, c[1].y, c[2].x, c[2].y, c[3].x, c[3].y, e);
    }
}

__global__ void __launch_bounds__(AK_LT) ak_flat_bwd_lane(ak_scene S, const float2 *__restrict__ ctrl,
                                                         const uint32_t *__restrict__ off, uint32_t cap,
                                                         const float2 *__restrict__ gpts,
                                                         float2 *__restrict__ gctrl) {
    const uint32_t s = blockIdx.x * AK_LT + threadIdx.x;
    if (s >= S.nseg || off[S.nseg] > cap)
        return;
    uint32_t     c0 = S.seg_cp[s], o = off[s];
    float2       p, c[4];
    ak_grad_emit e;
    e.g = gpts;
#pragma unroll
    for (int k = 0; k < 4; k++)
        e.gc[k] = make_float2(0.f, 0.f);
    if (seg_start(S, ctrl, s, p))
        e.gc[0] = gpts[o++];
    e.o              = o;
    const bool cubic = S.seg_kind[s] == AK_SEG_CUBIC;
    if (cubic && ak_cubic_cp(S, ctrl, s, c))
        gb_bezier_walk<true>(AK_TOL, c[0].x, c[0].y, c[1].x, c[1].y, c[2].x, c[2].y, c[3].x, c[3].y, e);
    atomicAdd(&gctrl[c0].x, e.gc[0].x), atomicAdd(&gctrl[c0].y, e.gc[0].y);
    if (cubic) {
        atomicAdd(&gctrl[c0 + 1].x, e.gc[1].x), atomicAdd(&gctrl[c0 + 1].y, e.gc[1].y);
        atomicAdd(&gctrl[c0 + 2].x, e.gc[2].x), atomicAdd(&gctrl[c0 + 2].y, e.gc[2].y);
        const uint32_t ce = S.seg_end[s];
        atomicAdd(&gctrl[ce].x, e.gc[3].x), atomicAdd(&gctrl[ce].y, e.gc[3].y);
    }
}

cudaError_t ak_launch_flat_count(cudaStream_t st, const ak_scene &S, const float2 *ctrl, uint32_t *cnt, bool lanes) {
    if (S.nseg && lanes)
        ak_flat_count_lane<<<(S.nseg + AK_LT - 1) / AK_LT, AK_LT, 0, st>>>(S, ctrl, cnt);
    else if (S.nseg)
        ak_flat_count<<<(S.nseg + AK_FW - 1) / AK_FW, 32 * AK_FW, 0, st>>>(S, ctrl, cnt);
    return cudaGetLastError();
}
cudaError_t ak_launch_flat_emit(cudaStream_t st, const ak_scene &S, const float2 *ctrl, const uint32_t *off,
                                float2 *pts, uint2 *pt_nb, uint32_t cap, uint32_t *status, bool lanes) {
    if (lanes)
        ak_flat_emit_lane<<<(S.nseg + AK_LT - 1) / AK_LT + 1, AK_LT, 0, st>>>(S, ctrl, off, pts, pt_nb, cap, status);
    else
        ak_flat_emit<<<(S.nseg + AK_FW - 1) / AK_FW + 1, 32 * AK_FW, 0, st>>>(S, ctrl, off, pts, pt_nb, cap, status);
    return cudaGetLastError();
}
cudaError_t ak_launch_flat_bwd(cudaStream_t st, const ak_scene &S, const float2 *ctrl, const uint32_t *off,
                               uint32_t cap, const float2 *gpts, float2 *gctrl, bool lanes) {
    if (S.nseg && lanes)
        ak_flat_bwd_lane<<<(S.nseg + AK_LT - 1) / AK_LT, AK_LT, 0, st>>>(S, ctrl, off, cap, gpts, gctrl);
    else if (S.nseg)
        ak_flat_bwd<<<(S.nseg + AK_FW - 1) / AK_FW, 32 * AK_FW, 0, st>>>(S, ctrl, off, cap, gpts, gctrl);
    return cudaGetLastError();
}
