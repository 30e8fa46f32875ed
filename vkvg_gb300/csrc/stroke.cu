/*
 * K2 - stroke expansion on sm_103a.
 *
 * Work items are "events": a join at a flattened point (vkvg's
 * _build_vb_step, src/vkvg_context_internal.c:924-1163), a start or end cap
 * (_draw_stoke_cap, :1165-1239), or the closing join of a closed subpath
 * (src/vkvg_context.c:917-932).  Undashed subpaths have one implicit event per
 * point, so every event is independent and runs in its own thread; dashed
 * subpaths are walked sequentially by one thread each (the dash phase is a
 * running fmodf carry, _draw_dashed_segment :1240-1264) and the walk writes an
 * explicit event list.  A count pass, a scan and an emit pass then produce
 * vkvg's own vertex and index buffers, with vertex indices relative to the
 * draw (vkvg's curVertOffset base).  A final pass applies vkvg's closed-path
 * index patch in subpath order.
 *
 * Built with -fmad=false and IEEE division/sqrt; trigonometry from pmath.h.
 */
#include "gb_types.h"
#include "pmath.h"

#include <cuda_runtime.h>
#include <float.h>

#define GB_PIF   3.14159265358979323846f
#define GB_PIF_2 1.57079632679489661923f

/* Iteration caps.  vkvg's round-join / round-cap loops never end when the arc
   step is 0 or negative (infinite or negative line width), and the dash walk
   never ends on an infinite segment; these caps bound the same loops here
   (and in the CPU restatement) far above any finite stroke's needs. */
#define GB_ARC_LOOP_CAP  65536u
#define GB_DASH_LOOP_CAP (1u << 22)

struct gb_sctx {
    float    hw, lh_max, arc_step;
    uint32_t join, cap;
};

__device__ __forceinline__ float2 v_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 v_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 v_mul(float2 a, float m) { return make_float2(a.x * m, a.y * m); }
__device__ __forceinline__ float2 v_div(float2 a, float m) { return make_float2(a.x / m, a.y / m); }
__device__ __forceinline__ float  v_len(float2 v) { return sqrtf(v.x * v.x + v.y * v.y); }
__device__ __forceinline__ float2 v_norm(float2 a) {
    float m = sqrtf(a.x * a.x + a.y * a.y);
    return make_float2(a.x / m, a.y / m);
}
__device__ __forceinline__ float2 v_perp(float2 a) { return make_float2(a.y, -a.x); }
__device__ __forceinline__ float  v_dot(float2 a, float2 b) { return (a.x * b.x) + (a.y * b.y); }
__device__ __forceinline__ bool   equf(float a, float b) { return fabsf(a - b) <= FLT_EPSILON; }
/* vec2_line_norm, src/vectors.h:103 */
__device__ __forceinline__ float2 v_line_norm(float2 a, float2 b) {
    float2 d  = make_float2(b.x - a.x, b.y - a.y);
    float  md = sqrtf(d.x * d.x + d.y * d.y);
    d.x /= md;
    d.y /= md;
    return d;
}

/* output sinks: count only, or write vertices/indices */
struct gb_count_out {
    uint32_t nv, ni, vbase;
    __device__ uint32_t idx() const { return vbase + nv; }
    __device__ void     vert(float2) { nv++; }
    __device__ void     tri(uint32_t, uint32_t, uint32_t) { ni += 3; }
};
struct gb_write_out {
    float2   *verts;
    uint32_t *inds;
    uint32_t  vo, io;     /* global write positions */
    uint32_t  vend, iend; /* this event's slots end here (from the count pass) */
    uint32_t  vrel;       /* draw-relative index of the next vertex */
    __device__ uint32_t idx() const { return vrel; }
    __device__ void     vert(float2 p) {
        if (vo < vend)
            verts[vo] = p;
        vo++;
        vrel++;
    }
    __device__ void tri(uint32_t a, uint32_t b, uint32_t c) {
        if (io + 3 <= iend) {
            inds[io]     = a;
            inds[io + 1] = b;
            inds[io + 2] = c;
        }
        io += 3;
    }
};

template <class O> __device__ __forceinline__ void rect_inds(O &o, uint32_t i) {
    o.tri(i, i + 2, i + 1);
    o.tri(i + 1, i + 2, i + 3);
}

/* _build_vb_step; returns det < 0 (or vkvg's specific return values) */
template <class O>
__device__ bool gb_build_vb_step(const float2 *__restrict__ pts, uint32_t cp, uint32_t iL, uint32_t iR, bool isCurve,
                                 const gb_sctx &s, O &o) {
    float2 p0        = pts[cp];
    float2 v0        = v_sub(p0, pts[iL]);
    float2 v1        = v_sub(pts[iR], p0);
    float  length_v0 = v_len(v0);
    float  length_v1 = v_len(v1);
    if (length_v0 < FLT_EPSILON || length_v1 < FLT_EPSILON)
        return false;
    float2 v0n = v_div(v0, length_v0);
    float2 v1n = v_div(v1, length_v1);
    float  dot = v_dot(v0n, v1n);
    float  det = v0n.x * v1n.y - v0n.y * v1n.x;
    if (equf(dot, 1.0f))
        return false;
    if (equf(dot, -1.0f)) {
        float2   vPerp = v_mul(v_perp(v0n), s.hw);
        uint32_t idx   = o.idx();
        o.vert(v_add(p0, vPerp));
        o.vert(v_sub(p0, vPerp));
        o.tri(idx, idx + 1, idx + 2);
        o.tri(idx, idx + 2, idx + 3);
        return true;
    }
    float2 bisec_n = v_norm(v_add(v0n, v1n));
    float  alpha   = pm_acosf(dot);
    if (det < 0)
        alpha = -alpha;
    float  halfAlpha    = alpha / 2.f;
    float  cosHalfAlpha = pm_cosf(halfAlpha);
    float  lh           = s.hw / cosHalfAlpha;
    float2 bisec_n_perp = v_perp(bisec_n);
    float  rlh          = lh;
    if (dot < 0.f)
        rlh = fminf(rlh, fminf(length_v0, length_v1));
    float2   bisec = v_mul(bisec_n_perp, rlh);
    uint32_t idx   = o.idx();
    float2   rlh_inside_pos, rlh_outside_pos;
    if (rlh < lh) {
        float2 vnPerp;
        if (length_v0 < length_v1)
            vnPerp = v_perp(v1n);
        else
            vnPerp = v_perp(v0n);
        float2 vHwPerp = v_mul(vnPerp, s.hw);
        float  lbc     = cosHalfAlpha * rlh;
        if (det < 0.f) {
            rlh_inside_pos  = v_add(v_add(v_mul(vnPerp, -lbc), v_add(p0, bisec)), vHwPerp);
            rlh_outside_pos = v_sub(p0, v_mul(bisec_n_perp, lh));
        } else {
            rlh_inside_pos  = v_sub(v_add(v_mul(vnPerp, lbc), v_sub(p0, bisec)), vHwPerp);
            rlh_outside_pos = v_add(p0, v_mul(bisec_n_perp, lh));
        }
    } else {
        if (det < 0.0f) {
            rlh_inside_pos  = v_add(p0, bisec);
            rlh_outside_pos = v_sub(p0, bisec);
        } else {
            rlh_inside_pos  = v_sub(p0, bisec);
            rlh_outside_pos = v_add(p0, bisec);
        }
    }
    uint32_t join = s.join;
    if (isCurve)
        join = dot < 0.8f ? 1u : 0u;
    if (join == 0u) {
        if (lh > s.lh_max) {
            float  x         = (lh - s.lh_max) * cosHalfAlpha;
            float2 bisecPerp = v_mul(bisec_n, x);
            bisec            = v_mul(bisec_n_perp, s.lh_max);
            if (det < 0) {
                o.vert(rlh_inside_pos);
                float2 p = v_sub(p0, bisec);
                o.vert(v_sub(p, bisecPerp));
                o.vert(v_add(p, bisecPerp));
                o.tri(idx, idx + 2, idx + 1);
                o.tri(idx + 2, idx + 4, idx);
                o.tri(idx, idx + 3, idx + 4);
                return true;
            } else {
                float2 p = v_add(p0, bisec);
                o.vert(v_sub(p, bisecPerp));
                o.vert(rlh_inside_pos);
                o.vert(v_add(p, bisecPerp));
                o.tri(idx, idx + 2, idx + 1);
                o.tri(idx + 2, idx + 3, idx + 1);
                o.tri(idx + 1, idx + 3, idx + 4);
                return false;
            }
        } else {
            if (det < 0) {
                o.vert(rlh_inside_pos);
                o.vert(rlh_outside_pos);
            } else {
                o.vert(rlh_outside_pos);
                o.vert(rlh_inside_pos);
            }
            rect_inds(o, idx);
            return false;
        }
    }
    float2 vp = v_perp(v0n);
    float2 pos;
    if (det < 0) {
        if (dot < 0 && rlh < lh)
            pos = rlh_inside_pos;
        else
            pos = v_add(p0, bisec);
        o.vert(pos);
        pos = v_sub(p0, v_mul(vp, s.hw));
    } else {
        o.vert(v_add(p0, v_mul(vp, s.hw)));
        if (dot < 0 && rlh < lh)
            pos = rlh_inside_pos;
        else
            pos = v_sub(p0, bisec);
    }
    o.vert(pos);
    if (join == 2u) {
        if (det < 0) {
            o.tri(idx, idx + 2, idx + 1);
            o.tri(idx + 2, idx + 4, idx + 0);
            o.tri(idx, idx + 3, idx + 4);
        } else {
            o.tri(idx, idx + 2, idx + 1);
            o.tri(idx + 2, idx + 3, idx + 1);
            o.tri(idx + 1, idx + 3, idx + 4);
        }
    } else if (join == 1u) {
        float a = pm_acosf(vp.x);
        if (vp.y < 0)
            a = -a;
        if (det < 0) {
            a += GB_PIF;
            float a1 = a + alpha;
            a -= s.arc_step;
            for (uint32_t it = 0; a > a1 && it < GB_ARC_LOOP_CAP; it++) {
                o.vert(make_float2(pm_cosf(a) * s.hw + p0.x, pm_sinf(a) * s.hw + p0.y));
                a -= s.arc_step;
            }
        } else {
            float a1 = a + alpha;
            a += s.arc_step;
            for (uint32_t it = 0; a < a1 && it < GB_ARC_LOOP_CAP; it++) {
                o.vert(make_float2(pm_cosf(a) * s.hw + p0.x, pm_sinf(a) * s.hw + p0.y));
                a += s.arc_step;
            }
        }
        uint32_t p0Idx = o.idx();
        o.tri(idx, idx + 2, idx + 1);
        if (det < 0) {
            for (uint32_t p = idx + 2; p < p0Idx; p++)
                o.tri(p, p + 1, idx);
            o.tri(p0Idx, p0Idx + 2, idx);
            o.tri(idx, p0Idx + 1, p0Idx + 2);
        } else {
            for (uint32_t p = idx + 2; p < p0Idx; p++)
                o.tri(p, p + 1, idx + 1);
            o.tri(p0Idx, p0Idx + 1, idx + 1);
            o.tri(idx + 1, p0Idx + 1, p0Idx + 2);
        }
    }
    vp = v_mul(v_perp(v1n), s.hw);
    if (det < 0)
        o.vert(v_sub(p0, vp));
    else
        o.vert(v_add(p0, vp));
    return det < 0;
}

/* _draw_stoke_cap */
template <class O> __device__ void gb_draw_cap(float2 p0, float2 n, bool isStart, const gb_sctx &s, O &o) {
    uint32_t firstIdx = o.idx();
    if (isStart) {
        float2 vhw = v_mul(n, s.hw);
        if (s.cap == 2u)
            p0 = v_sub(p0, vhw);
        vhw = v_perp(vhw);
        if (s.cap == 1u) {
            float a = pm_acosf(n.x) + GB_PIF_2;
            if (n.y < 0)
                a = GB_PIF - a;
            float a1 = a + GB_PIF;
            a += s.arc_step;
            for (uint32_t it = 0; a < a1 && it < GB_ARC_LOOP_CAP; it++) {
                o.vert(make_float2(pm_cosf(a) * s.hw + p0.x, pm_sinf(a) * s.hw + p0.y));
                a += s.arc_step;
            }
            uint32_t p0Idx = o.idx();
            for (uint32_t p = firstIdx; p < p0Idx; p++)
                o.tri(p0Idx + 1, p, p + 1);
            firstIdx = p0Idx;
        }
        o.vert(v_add(p0, vhw));
        o.vert(v_sub(p0, vhw));
        rect_inds(o, firstIdx);
    } else {
        float2 vhw = v_mul(n, s.hw);
        if (s.cap == 2u)
            p0 = v_add(p0, vhw);
        vhw = v_perp(vhw);
        o.vert(v_add(p0, vhw));
        o.vert(v_sub(p0, vhw));
        firstIdx = o.idx();
        if (s.cap == 1u) {
            float a = pm_acosf(n.x) + GB_PIF_2;
            if (n.y < 0)
                a = GB_PIF - a;
            float a1 = a - GB_PIF;
            a -= s.arc_step;
            for (uint32_t it = 0; a > a1 && it < GB_ARC_LOOP_CAP; it++) {
                o.vert(make_float2(pm_cosf(a) * s.hw + p0.x, pm_sinf(a) * s.hw + p0.y));
                a -= s.arc_step;
            }
            uint32_t p0Idx = o.idx() - 1;
            for (uint32_t p = firstIdx - 1; p < p0Idx; p++)
                o.tri(p + 1, p, firstIdx - 2);
        }
    }
}

__device__ __forceinline__ gb_sctx make_sctx(const gb_draw &d) {
    gb_sctx s;
    s.hw       = d.hw;
    s.lh_max   = d.lh_max;
    s.arc_step = d.arc_step;
    s.join     = d.join;
    s.cap      = d.cap;
    return s;
}

/* ------------------------------------------------------------ dash walk */

/* Sequential walk of a dashed subpath (_stroke_preserve with dashCount > 0,
   src/vkvg_context.c:853-916).  Writes events when ev != nullptr; returns the
   event count.  The end-of-dash read of dashes[-1] in vkvg (curDash == 0) is
   replaced by the last dash entry. */
__device__ uint32_t gb_dash_walk(const float2 *__restrict__ pts, const uint8_t *__restrict__ pflag, uint32_t first,
                                 uint32_t n, bool closed, const float *__restrict__ dashes, uint32_t dcount,
                                 float doffset, gb_event *ev, uint32_t ev_cap) {
    float tot = 0;
    for (uint32_t i = 0; i < dcount; i++)
        tot += dashes[i];
    bool     dashOn  = true;
    uint32_t curDash = 0;
    float    curOff  = fmodf(doffset, tot);
    float2   normal  = make_float2(0, 0);
    uint32_t ne      = 0;
    uint32_t last    = first + n - 1;
    uint32_t iL = last, cp = first, iR = first;
    auto segment = [&](uint32_t cpi, uint32_t iLi, uint32_t iRi, bool curved) {
        float2 p  = pts[cpi];
        float2 pR = pts[iRi];
        if (!dashOn) {
            if (ev && ne < ev_cap)
                ev[ne] = {GB_EV_JOIN | (curved ? 0x100u : 0u), cpi, iLi, iRi, 0, 0, 0, 0};
            ne++;
        }
        float2 d      = v_sub(pR, p);
        normal        = v_norm(d);
        float seglen  = v_len(d);
        while (curOff < seglen && ne < GB_DASH_LOOP_CAP) {
            float2 p0 = v_add(p, v_mul(normal, curOff));
            if (ev && ne < ev_cap)
                ev[ne] = {dashOn ? GB_EV_CAP_START : GB_EV_CAP_END, 0, 0, 0, p0.x, p0.y, normal.x, normal.y};
            ne++;
            dashOn = !dashOn;
            curOff += dashes[curDash];
            if (++curDash == dcount)
                curDash = 0;
        }
        curOff -= seglen;
        curOff = fmodf(curOff, tot);
    };
    while (cp < last) {
        iR = cp + 1;
        segment(cp, iL, iR, pflag[cp] != 0);
        iL = cp++;
    }
    if (closed) {
        iR = first;
        segment(cp, iL, iR, false);
    }
    if (!dashOn) {
        int32_t prevDash = (int32_t)curDash - 1;
        if (prevDash < 0) {
            curDash  = dcount - 1;
            prevDash = (int32_t)dcount - 1;
        }
        float  m = fminf(dashes[prevDash] - curOff, dashes[curDash]);
        float2 p = v_sub(pts[iR], v_mul(normal, m));
        if (ev && ne < ev_cap)
            ev[ne] = {GB_EV_CAP_END, 0, 0, 0, p.x, p.y, normal.x, normal.y};
        ne++;
    }
    return ne;
}

/* events per stroke (draw, subpath) pair */
__global__ void gb_stroke_pair_events(uint32_t npairs, const uint32_t *__restrict__ pair_draw,
                                      const uint32_t *__restrict__ pair_sub, const gb_draw *__restrict__ draws,
                                      const uint32_t *__restrict__ sub_pt0, const uint32_t *__restrict__ sub_npts,
                                      const uint32_t *__restrict__ sub_flags, const float2 *__restrict__ pts,
                                      const uint8_t *__restrict__ pflag, const float *__restrict__ dashes,
                                      uint32_t *__restrict__ counts, int walk_dashes) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs)
        return;
    const gb_draw &d = draws[pair_draw[p]];
    uint32_t       s = pair_sub[p];
    uint32_t       n = sub_npts[s];
    if (n < 2) {
        counts[p] = 0;
        return;
    }
    if (d.dash_count == 0) {
        counts[p] = n;
        return;
    }
    if (!walk_dashes)
        return; /* counted by gb_dash_state */
    counts[p] = gb_dash_walk(pts, pflag, sub_pt0[s], n, (sub_flags[s] & GB_SUB_CLOSED) != 0, dashes + d.dash_first,
                             d.dash_count, d.dash_offset, nullptr, 0);
}
/* materialise dashed events */
__global__ void gb_stroke_dash_events(uint32_t npairs, const uint32_t *__restrict__ pair_draw,
                                      const uint32_t *__restrict__ pair_sub, const gb_draw *__restrict__ draws,
                                      const uint32_t *__restrict__ sub_pt0, const uint32_t *__restrict__ sub_npts,
                                      const uint32_t *__restrict__ sub_flags, const float2 *__restrict__ pts,
                                      const uint8_t *__restrict__ pflag, const float *__restrict__ dashes,
                                      const uint32_t *__restrict__ ev_off, gb_event *__restrict__ events) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs)
        return;
    const gb_draw &d = draws[pair_draw[p]];
    uint32_t       s = pair_sub[p];
    uint32_t       n = sub_npts[s];
    if (n < 2 || d.dash_count == 0)
        return;
    gb_dash_walk(pts, pflag, sub_pt0[s], n, (sub_flags[s] & GB_SUB_CLOSED) != 0, dashes + d.dash_first, d.dash_count,
                 d.dash_offset, events + ev_off[p], ev_off[p + 1] - ev_off[p]);
}

/* ---- dashed subpaths in parallel.
 *
 * The same computation as gb_dash_walk in three steps: (A) every segment's
 * length, in parallel; (B) per dashed pair, only the sequential dash
 * recurrence over those lengths, recording at each segment's first point the
 * dash state entering it, its event offset within the pair and its number of
 * dash boundaries; (C) every segment's events replayed from that state, in
 * parallel.  Each float operation is the one gb_dash_walk performs, in the
 * same order, so the events are identical.  The per-point records require
 * that no subpath belongs to two dashed pairs of one frame (the host falls
 * back to gb_dash_walk otherwise). */
__global__ void gb_dash_seglen(uint32_t npairs, const uint32_t *__restrict__ pair_draw,
                               const uint32_t *__restrict__ pair_sub, const gb_draw *__restrict__ draws,
                               const uint32_t *__restrict__ sub_pt0, const uint32_t *__restrict__ sub_npts,
                               const uint32_t *__restrict__ sub_flags, const float2 *__restrict__ pts,
                               float *__restrict__ seglen) {
    const uint32_t p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (p >= npairs)
        return;
    const gb_draw &d = draws[pair_draw[p]];
    const uint32_t s = pair_sub[p], n = sub_npts[s];
    if (n < 2 || d.dash_count == 0)
        return;
    const uint32_t first = sub_pt0[s];
    const uint32_t nseg  = n - 1 + ((sub_flags[s] & GB_SUB_CLOSED) ? 1u : 0u);
    for (uint32_t j = lane; j < nseg; j += 32) {
        const uint32_t cp = first + j, iR = j < n - 1 ? cp + 1 : first;
        seglen[cp]        = v_len(v_sub(pts[iR], pts[cp]));
    }
}
/* dash entry i of a pattern held in registers (patterns of up to 4 entries) */
__device__ __forceinline__ float dash_at(const float (&dr)[4], uint32_t i) {
    return i == 0 ? dr[0] : i == 1 ? dr[1] : i == 2 ? dr[2] : dr[3];
}
template <bool REG>
__device__ __forceinline__ void dash_state_walk(const float *__restrict__ dashes, uint32_t dcount, float doffset,
                                                uint32_t first, uint32_t nseg, const float *__restrict__ seglen,
                                                uint4 *__restrict__ dseg, uint4 *__restrict__ fin_out,
                                                uint32_t *__restrict__ count_out) {
    float dr[4] = {0, 0, 0, 0};
    if (REG)
        for (uint32_t i = 0; i < dcount; i++)
            dr[i == 0 ? 0 : i == 1 ? 1 : i == 2 ? 2 : 3] = dashes[i];
    float tot = 0;
    for (uint32_t i = 0; i < dcount; i++)
        tot += dashes[i];
    bool        dashOn  = true;
    uint32_t    curDash = 0;
    float       curOff  = fmodf(doffset, tot);
    uint32_t    ne      = 0;
    const float atot    = fabsf(tot);
    float       dv      = REG ? dr[0] : dashes[0]; /* dashes[curDash] */
    /* lengths are read 16 at a time so that their latency is paid once per
       16 segments; the recurrence itself is strictly sequential */
    for (uint32_t j0 = 0; j0 < nseg; j0 += 16) {
        float sl16[16];
#pragma unroll
        for (int q = 0; q < 16; q++)
            sl16[q] = j0 + q < nseg ? seglen[first + j0 + q] : 0.f;
#pragma unroll
        for (int q = 0; q < 16; q++) {
            if (j0 + q >= nseg)
                break;
            const uint32_t cp  = first + j0 + q;
            const float    sl  = sl16[q];
            uint4          rec = make_uint4(__float_as_uint(curOff), curDash | (dashOn ? 0x80000000u : 0u), ne, 0);
            if (!dashOn)
                ne++; /* the segment's join */
            uint32_t k = 0;
            while (curOff < sl && ne < GB_DASH_LOOP_CAP) {
                ne++;
                dashOn = !dashOn;
                curOff += dv; /* dashes[curDash] */
                if (++curDash == dcount)
                    curDash = 0;
                dv = REG ? dash_at(dr, curDash) : dashes[curDash]; /* next entry, off the add chain */
                k++;
            }
            curOff -= sl;
            if (!(fabsf(curOff) < atot)) /* fmodf(x, t) is x itself when |x| < |t| */
                curOff = fmodf(curOff, tot);
            rec.w    = k;
            dseg[cp] = rec;
        }
    }
    const uint32_t total = ne + (dashOn ? 0u : 1u);
    *fin_out   = make_uint4(__float_as_uint(curOff), curDash | (dashOn ? 0x80000000u : 0u), total, 0);
    *count_out = total;
}
__global__ void gb_dash_state(uint32_t npairs, const uint32_t *__restrict__ pair_draw,
                              const uint32_t *__restrict__ pair_sub, const gb_draw *__restrict__ draws,
                              const uint32_t *__restrict__ sub_pt0, const uint32_t *__restrict__ sub_npts,
                              const uint32_t *__restrict__ sub_flags, const float *__restrict__ dash_arr,
                              const float *__restrict__ seglen, uint4 *__restrict__ dseg, uint4 *__restrict__ dfin,
                              uint32_t *__restrict__ counts) {
    /* one warp per pair, lane 0 walking: pairs of one warp would serialise
       each other's divergent boundary loops */
    const uint32_t p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (p >= npairs || (threadIdx.x & 31) != 0)
        return;
    const gb_draw &d = draws[pair_draw[p]];
    const uint32_t s = pair_sub[p], n = sub_npts[s];
    if (n < 2 || d.dash_count == 0)
        return;
    const uint32_t nseg = n - 1 + ((sub_flags[s] & GB_SUB_CLOSED) ? 1u : 0u);
    if (d.dash_count <= 4)
        dash_state_walk<true>(dash_arr + d.dash_first, d.dash_count, d.dash_offset, sub_pt0[s], nseg, seglen, dseg,
                              dfin + p, counts + p);
    else
        dash_state_walk<false>(dash_arr + d.dash_first, d.dash_count, d.dash_offset, sub_pt0[s], nseg, seglen, dseg,
                               dfin + p, counts + p);
}
__global__ void gb_dash_emit(uint32_t npairs, const uint32_t *__restrict__ pair_draw,
                             const uint32_t *__restrict__ pair_sub, const gb_draw *__restrict__ draws,
                             const uint32_t *__restrict__ sub_pt0, const uint32_t *__restrict__ sub_npts,
                             const uint32_t *__restrict__ sub_flags, const float2 *__restrict__ pts,
                             const uint8_t *__restrict__ pflag, const float *__restrict__ dash_arr,
                             const uint4 *__restrict__ dseg, const uint4 *__restrict__ dfin,
                             const uint32_t *__restrict__ ev_off, gb_event *__restrict__ events) {
    const uint32_t p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (p >= npairs)
        return;
    const gb_draw &d = draws[pair_draw[p]];
    const uint32_t s = pair_sub[p], n = sub_npts[s];
    if (n < 2 || d.dash_count == 0)
        return;
    const float   *dashes = dash_arr + d.dash_first;
    const uint32_t dcount = d.dash_count;
    const uint32_t first = sub_pt0[s], last = first + n - 1;
    const uint32_t nseg  = n - 1 + ((sub_flags[s] & GB_SUB_CLOSED) ? 1u : 0u);
    gb_event      *ev    = events + ev_off[p];
    const uint32_t cap   = ev_off[p + 1] - ev_off[p];
    for (uint32_t j = lane; j < nseg; j += 32) {
        const uint32_t cp = first + j, iR = j < n - 1 ? cp + 1 : first, iL = j == 0 ? last : cp - 1;
        const bool     curved  = j < n - 1 ? pflag[cp] != 0 : false;
        const uint4    rec     = dseg[cp];
        float          curOff  = __uint_as_float(rec.x);
        uint32_t       curDash = rec.y & 0x7FFFFFFFu;
        bool           dashOn  = (rec.y >> 31) != 0;
        uint32_t       e       = rec.z;
        if (!dashOn) {
            if (e < cap)
                ev[e] = {GB_EV_JOIN | (curved ? 0x100u : 0u), cp, iL, iR, 0, 0, 0, 0};
            e++;
        }
        const float2 pc     = pts[cp];
        const float2 normal = v_norm(v_sub(pts[iR], pc));
        for (uint32_t k = 0; k < rec.w; k++) {
            const float2 p0 = v_add(pc, v_mul(normal, curOff));
            if (e < cap)
                ev[e] = {dashOn ? GB_EV_CAP_START : GB_EV_CAP_END, 0, 0, 0, p0.x, p0.y, normal.x, normal.y};
            e++;
            dashOn = !dashOn;
            curOff += dashes[curDash];
            if (++curDash == dcount)
                curDash = 0;
        }
    }
    if (lane == 0) {
        const uint4 fin = dfin[p];
        if ((fin.y >> 31) == 0) { /* the dash is still on: close it at the end */
            const float    curOff  = __uint_as_float(fin.x);
            uint32_t       curDash = fin.y & 0x7FFFFFFFu;
            const uint32_t cpl = first + nseg - 1, iRl = nseg - 1 < n - 1 ? cpl + 1 : first;
            const float2   normal  = v_norm(v_sub(pts[iRl], pts[cpl]));
            int32_t        prevDash = (int32_t)curDash - 1;
            if (prevDash < 0) {
                curDash  = dcount - 1;
                prevDash = (int32_t)dcount - 1;
            }
            const float  m  = fminf(dashes[prevDash] - curOff, dashes[curDash]);
            const float2 pe = v_sub(pts[iRl], v_mul(normal, m));
            if (fin.z - 1 < cap)
                ev[fin.z - 1] = {GB_EV_CAP_END, 0, 0, 0, pe.x, pe.y, normal.x, normal.y};
        }
    }
}

/* locate the pair of a global event index */
__device__ __forceinline__ uint32_t find_pair(const uint32_t *__restrict__ ev_off, uint32_t npairs, uint32_t e) {
    uint32_t lo = 0, hi = npairs; /* ev_off[lo] <= e < ev_off[hi] */
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (ev_off[mid] <= e)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

/* decode the event e (global) into a concrete event */
__device__ __forceinline__ gb_event decode_event(uint32_t e, uint32_t p, const uint32_t *__restrict__ ev_off,
                                                 const gb_draw &d, uint32_t first, uint32_t n, bool closed,
                                                 const float2 *__restrict__ pts, const uint8_t *__restrict__ pflag,
                                                 const gb_event *__restrict__ events) {
    if (d.dash_count > 0)
        return events[e];
    uint32_t j    = e - ev_off[p];
    uint32_t last = first + n - 1;
    gb_event ev;
    ev.px = ev.py = ev.nx = ev.ny = 0;
    if (!closed) {
        if (j == 0) {
            float2 nn = v_line_norm(pts[first], pts[first + 1]);
            float2 pp = pts[first];
            ev        = {GB_EV_CAP_START, 0, 0, 0, pp.x, pp.y, nn.x, nn.y};
            return ev;
        }
        if (j == n - 1) {
            float2 nn = v_line_norm(pts[last - 1], pts[last]);
            float2 pp = pts[last];
            ev        = {GB_EV_CAP_END, 0, 0, 0, pp.x, pp.y, nn.x, nn.y};
            return ev;
        }
        uint32_t cp = first + j;
        ev          = {GB_EV_JOIN | (pflag[cp] ? 0x100u : 0u), cp, cp - 1, cp + 1, 0, 0, 0, 0};
        return ev;
    }
    if (j == n - 1) {
        ev = {GB_EV_CLOSE, last, last - 1, first, 0, 0, 0, 0};
        return ev;
    }
    uint32_t cp = first + j;
    ev          = {GB_EV_JOIN | (pflag[cp] ? 0x100u : 0u), cp, j == 0 ? last : cp - 1, cp + 1, 0, 0, 0, 0};
    return ev;
}

template <class O>
__device__ __forceinline__ bool run_event(const gb_event &ev, const float2 *__restrict__ pts, const gb_sctx &s, O &o) {
    uint32_t k = ev.kind & 0xFFu;
    if (k == GB_EV_JOIN)
        return gb_build_vb_step(pts, ev.cp, ev.iL, ev.iR, (ev.kind & 0x100u) != 0, s, o);
    if (k == GB_EV_CLOSE)
        return gb_build_vb_step(pts, ev.cp, ev.iL, ev.iR, false, s, o);
    if (k == GB_EV_CAP_START || k == GB_EV_CAP_END)
        gb_draw_cap(make_float2(ev.px, ev.py), make_float2(ev.nx, ev.ny), k == GB_EV_CAP_START, s, o);
    return false;
}

/* per-event vertex and index counts */
__global__ void gb_stroke_event_count(uint32_t nev, uint32_t npairs, const uint32_t *__restrict__ ev_off,
                                      const uint32_t *__restrict__ pair_draw, const uint32_t *__restrict__ pair_sub,
                                      const gb_draw *__restrict__ draws, const uint32_t *__restrict__ sub_pt0,
                                      const uint32_t *__restrict__ sub_npts, const uint32_t *__restrict__ sub_flags,
                                      const float2 *__restrict__ pts, const uint8_t *__restrict__ pflag,
                                      const gb_event *__restrict__ events, uint32_t *__restrict__ cnt_v,
                                      uint32_t *__restrict__ cnt_i) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nev)
        return;
    uint32_t       p = find_pair(ev_off, npairs, e);
    const gb_draw &d = draws[pair_draw[p]];
    uint32_t       s = pair_sub[p];
    gb_event ev = decode_event(e, p, ev_off, d, sub_pt0[s], sub_npts[s], (sub_flags[s] & GB_SUB_CLOSED) != 0, pts,
                               pflag, events);
    gb_sctx      sc = make_sctx(d);
    gb_count_out o{0, 0, 0};
    run_event(ev, pts, sc, o);
    cnt_v[e] = o.nv;
    cnt_i[e] = o.ni;
}

/* emission at the scanned offsets; pair_dfirst[p] = first pair of p's draw,
   whose first vertex is the draw's vertex base */
__global__ void gb_stroke_event_emit(uint32_t nev, uint32_t npairs, const uint32_t *__restrict__ ev_off,
                                     const uint32_t *__restrict__ pair_draw, const uint32_t *__restrict__ pair_sub,
                                     const gb_draw *__restrict__ draws, const uint32_t *__restrict__ sub_pt0,
                                     const uint32_t *__restrict__ sub_npts, const uint32_t *__restrict__ sub_flags,
                                     const float2 *__restrict__ pts, const uint8_t *__restrict__ pflag,
                                     const gb_event *__restrict__ events, const uint32_t *__restrict__ off_v,
                                     const uint32_t *__restrict__ off_i, const uint32_t *__restrict__ pair_dfirst,
                                     float2 *__restrict__ verts, uint32_t *__restrict__ inds,
                                     uint8_t *__restrict__ ev_ret) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nev)
        return;
    uint32_t       p = find_pair(ev_off, npairs, e);
    const gb_draw &d = draws[pair_draw[p]];
    uint32_t       s = pair_sub[p];
    gb_event ev = decode_event(e, p, ev_off, d, sub_pt0[s], sub_npts[s], (sub_flags[s] & GB_SUB_CLOSED) != 0, pts,
                               pflag, events);
    gb_sctx      sc = make_sctx(d);
    uint32_t     vbase = off_v[ev_off[pair_dfirst[p]]];
    gb_write_out o{verts, inds, off_v[e], off_i[e], off_v[e + 1], off_i[e + 1], off_v[e] - vbase};
    ev_ret[e] = run_event(ev, pts, sc, o) ? 1 : 0;
}

/* vkvg's closed-path patch of the last six indices (src/vkvg_context.c:917-932),
   applied in subpath order, one thread per stroke draw; limited to the draw's
   own indices. */
__global__ void gb_stroke_close_patch(uint32_t ndraw_s, const uint32_t *__restrict__ draw_pair0,
                                      const uint32_t *__restrict__ pair_sub, const gb_draw *__restrict__ draws,
                                      const uint32_t *__restrict__ pair_draw, const uint32_t *__restrict__ sub_npts,
                                      const uint32_t *__restrict__ sub_flags, const uint32_t *__restrict__ ev_off,
                                      const uint32_t *__restrict__ off_v, const uint32_t *__restrict__ off_i,
                                      const uint8_t *__restrict__ ev_ret, uint32_t *__restrict__ inds) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ndraw_s)
        return;
    uint32_t p0 = draw_pair0[k], p1 = draw_pair0[k + 1];
    if (p0 == p1)
        return;
    const gb_draw &d = draws[pair_draw[p0]];
    if (d.dash_count > 0)
        return;
    uint32_t ibase = off_i[ev_off[p0]], vbase = off_v[ev_off[p0]];
    for (uint32_t p = p0; p < p1; p++) {
        uint32_t s = pair_sub[p];
        if (!(sub_flags[s] & GB_SUB_CLOSED) || sub_npts[s] < 2)
            continue;
        uint32_t eclose = ev_off[p + 1] - 1; /* the closing join */
        uint32_t iend   = off_i[eclose + 1];
        if (iend - ibase < 6)
            continue;
        uint32_t *ix  = inds + iend - 6;
        uint32_t  ii  = off_v[ev_off[p]] - vbase; /* str.firstIdx */
        if (ev_ret[eclose]) {
            ix[1] = ii + 1;
            ix[4] = ii + 1;
            ix[5] = ii;
        } else {
            ix[1] = ii;
            ix[4] = ii;
            ix[5] = ii + 1;
        }
    }
}

/* per stroke draw: first triangle and first vertex in the global buffers */
__global__ void gb_stroke_draw_bases(uint32_t ndraw_s, const uint32_t *__restrict__ draw_pair0,
                                     const uint32_t *__restrict__ ev_off, const uint32_t *__restrict__ off_v,
                                     const uint32_t *__restrict__ off_i, uint32_t *__restrict__ draw_tri0,
                                     uint32_t *__restrict__ draw_vbase) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > ndraw_s)
        return;
    uint32_t e    = ev_off[draw_pair0[k]];
    draw_tri0[k]  = off_i[e] / 3;
    draw_vbase[k] = off_v[e];
}

extern "C" {
cudaError_t gb_launch_stroke_draw_bases(cudaStream_t st, uint32_t ndraw_s, const uint32_t *draw_pair0,
                                        const uint32_t *ev_off, const uint32_t *off_v, const uint32_t *off_i,
                                        uint32_t *draw_tri0, uint32_t *draw_vbase) {
    gb_stroke_draw_bases<<<(ndraw_s + 1 + 127) / 128, 128, 0, st>>>(ndraw_s, draw_pair0, ev_off, off_v, off_i,
                                                                      draw_tri0, draw_vbase);
    return cudaGetLastError();
}
cudaError_t gb_launch_stroke_pair_events(cudaStream_t st, uint32_t npairs, const uint32_t *pair_draw,
                                         const uint32_t *pair_sub, const gb_draw *draws, const uint32_t *sub_pt0,
                                         const uint32_t *sub_npts, const uint32_t *sub_flags, const float2 *pts,
                                         const uint8_t *pflag, const float *dashes, uint32_t *counts,
                                         int walk_dashes) {
    if (!npairs)
        return cudaSuccess;
    gb_stroke_pair_events<<<(npairs + 127) / 128, 128, 0, st>>>(npairs, pair_draw, pair_sub, draws, sub_pt0, sub_npts,
                                                                 sub_flags, pts, pflag, dashes, counts, walk_dashes);
    return cudaGetLastError();
}
cudaError_t gb_launch_dash_count(cudaStream_t st, uint32_t npairs, const uint32_t *pair_draw, const uint32_t *pair_sub,
                                 const gb_draw *draws, const uint32_t *sub_pt0, const uint32_t *sub_npts,
                                 const uint32_t *sub_flags, const float2 *pts, const float *dashes, float *seglen,
                                 uint4 *dseg, uint4 *dfin, uint32_t *counts) {
    if (!npairs)
        return cudaSuccess;
    gb_dash_seglen<<<(npairs + 7) / 8, 256, 0, st>>>(npairs, pair_draw, pair_sub, draws, sub_pt0, sub_npts, sub_flags,
                                                      pts, seglen);
    gb_dash_state<<<(npairs + 3) / 4, 128, 0, st>>>(npairs, pair_draw, pair_sub, draws, sub_pt0, sub_npts, sub_flags,
                                                      dashes, seglen, dseg, dfin, counts);
    return cudaGetLastError();
}
cudaError_t gb_launch_dash_emit(cudaStream_t st, uint32_t npairs, const uint32_t *pair_draw, const uint32_t *pair_sub,
                                const gb_draw *draws, const uint32_t *sub_pt0, const uint32_t *sub_npts,
                                const uint32_t *sub_flags, const float2 *pts, const uint8_t *pflag,
                                const float *dashes, const uint4 *dseg, const uint4 *dfin, const uint32_t *ev_off,
                                gb_event *events) {
    if (!npairs)
        return cudaSuccess;
    gb_dash_emit<<<(npairs + 7) / 8, 256, 0, st>>>(npairs, pair_draw, pair_sub, draws, sub_pt0, sub_npts, sub_flags,
                                                    pts, pflag, dashes, dseg, dfin, ev_off, events);
    return cudaGetLastError();
}
cudaError_t gb_launch_stroke_dash_events(cudaStream_t st, uint32_t npairs, const uint32_t *pair_draw,
                                         const uint32_t *pair_sub, const gb_draw *draws, const uint32_t *sub_pt0,
                                         const uint32_t *sub_npts, const uint32_t *sub_flags, const float2 *pts,
                                         const uint8_t *pflag, const float *dashes, const uint32_t *ev_off,
                                         gb_event *events) {
    if (!npairs)
        return cudaSuccess;
    gb_stroke_dash_events<<<(npairs + 127) / 128, 128, 0, st>>>(npairs, pair_draw, pair_sub, draws, sub_pt0, sub_npts,
                                                                 sub_flags, pts, pflag, dashes, ev_off, events);
    return cudaGetLastError();
}
cudaError_t gb_launch_stroke_event_count(cudaStream_t st, uint32_t nev, uint32_t npairs, const uint32_t *ev_off,
                                         const uint32_t *pair_draw, const uint32_t *pair_sub, const gb_draw *draws,
                                         const uint32_t *sub_pt0, const uint32_t *sub_npts, const uint32_t *sub_flags,
                                         const float2 *pts, const uint8_t *pflag, const gb_event *events,
                                         uint32_t *cnt_v, uint32_t *cnt_i) {
    if (!nev)
        return cudaSuccess;
    gb_stroke_event_count<<<(nev + 127) / 128, 128, 0, st>>>(nev, npairs, ev_off, pair_draw, pair_sub, draws, sub_pt0,
                                                              sub_npts, sub_flags, pts, pflag, events, cnt_v, cnt_i);
    return cudaGetLastError();
}
cudaError_t gb_launch_stroke_event_emit(cudaStream_t st, uint32_t nev, uint32_t npairs, const uint32_t *ev_off,
                                        const uint32_t *pair_draw, const uint32_t *pair_sub, const gb_draw *draws,
                                        const uint32_t *sub_pt0, const uint32_t *sub_npts, const uint32_t *sub_flags,
                                        const float2 *pts, const uint8_t *pflag, const gb_event *events,
                                        const uint32_t *off_v, const uint32_t *off_i, const uint32_t *pair_dfirst,
                                        float2 *verts, uint32_t *inds, uint8_t *ev_ret) {
    if (!nev)
        return cudaSuccess;
    gb_stroke_event_emit<<<(nev + 127) / 128, 128, 0, st>>>(nev, npairs, ev_off, pair_draw, pair_sub, draws, sub_pt0,
                                                             sub_npts, sub_flags, pts, pflag, events, off_v, off_i,
                                                             pair_dfirst, verts, inds, ev_ret);
    return cudaGetLastError();
}
cudaError_t gb_launch_stroke_close_patch(cudaStream_t st, uint32_t ndraw_s, const uint32_t *draw_pair0,
                                         const uint32_t *pair_sub, const gb_draw *draws, const uint32_t *pair_draw,
                                         const uint32_t *sub_npts, const uint32_t *sub_flags, const uint32_t *ev_off,
                                         const uint32_t *off_v, const uint32_t *off_i, const uint8_t *ev_ret,
                                         uint32_t *inds) {
    if (!ndraw_s)
        return cudaSuccess;
    gb_stroke_close_patch<<<(ndraw_s + 127) / 128, 128, 0, st>>>(ndraw_s, draw_pair0, pair_sub, draws, pair_draw,
                                                                  sub_npts, sub_flags, ev_off, off_v, off_i, ev_ret,
                                                                  inds);
    return cudaGetLastError();
}
}
