/*
 * vkvg's cubic flattening, _recursive_bezier (src/vkvg_context_internal.c:
 * 1313-1461, AGG adaptive subdivision), as an explicit-stack depth-first walk
 * that visits the points in exactly the order of the recursive host code.
 * Shared by the plain flatten kernels and the analytic-coverage kernels.
 *
 * Every emitted point is one of three points of the current sub-curve:
 * its midpoint x1234 (GB_BEZ_MID), its second control point x2 (GB_BEZ_C2)
 * or its third x3 (GB_BEZ_C3).  With TRACK the walk also carries the
 * sub-curve's parameter interval [ta, tb] on the original cubic, so a caller
 * can express the point as a fixed linear combination of the four control
 * points (the blossom of the interval); without TRACK ta = tb = 0.
 *
 * Units that include this file are built with -fmad=false and IEEE division
 * so that every decision matches the CPU restatement bit for bit.  vkvg
 * compares float values against the double constants 1.7 and 0.01; the float
 * forms below are the exact equivalents:
 *     d > 1.7 (double)   <=>  d >= 1.7f        (1.7f > 1.7 > prev(1.7f))
 *     d < 0.01 (double)  <=>  d <= 0.01f       (0.01f < 0.01 < next(0.01f))
 *     d > 0.01 (double)  <=>  d >  0.01f
 */
#pragma once
#include "pmath.h"

#define GB_PIF  3.14159265358979323846f
#define GB_2PIF 0.63661977236758134308f /* vkvg's M_2_PIF = 2/pi (src/vkvg_internal.h:45) */

/* work cap per cubic: far above any finite curve's subdivision tree */
#define GB_CURVE_NODE_CAP (1u << 22)

#define GB_BEZ_MID 0
#define GB_BEZ_C2  1
#define GB_BEZ_C3  2

struct gb_bez_frame {
    float x1, y1, x2, y2, x3, y3, x4, y4;
    unsigned level;
};

/* What one node of the subdivision tree does: add n (1 or 2) points and
   stop, or (sub) split into its two halves, whose control points are
   (x1, x12, x123, x1234) and (x1234, x234, x34, x4). */
struct gb_bez_step {
    int    n, w0, w1; /* points added and which sub-curve points they are */
    float2 p0, p1;
    bool   sub;
    float  x12, y12, x123, y123, x1234, y1234, x234, y234, x34, y34;
};

/* _recursive_bezier's test at one node (src/vkvg_context_internal.c:
   1320-1455), the same float operations in the same order */
__device__ __forceinline__ void gb_bez_eval(float tol, const gb_bez_frame &f, gb_bez_step &s) {
    s.n = 0, s.sub = false;
    s.x12   = (f.x1 + f.x2) / 2;
    s.y12   = (f.y1 + f.y2) / 2;
    float x23 = (f.x2 + f.x3) / 2;
    float y23 = (f.y2 + f.y3) / 2;
    s.x34   = (f.x3 + f.x4) / 2;
    s.y34   = (f.y3 + f.y4) / 2;
    s.x123  = (s.x12 + x23) / 2;
    s.y123  = (s.y12 + y23) / 2;
    s.x234  = (x23 + s.x34) / 2;
    s.y234  = (y23 + s.y34) / 2;
    s.x1234 = (s.x123 + s.x234) / 2;
    s.y1234 = (s.y123 + s.y234) / 2;
#define GB_EMIT1(px, py, w)                                                                                             \
    {                                                                                                                  \
        s.n = 1, s.p0 = make_float2(px, py), s.w0 = w;                                                                 \
        return;                                                                                                        \
    }
    if (f.level > 0u) {
        float dx = f.x4 - f.x1;
        float dy = f.y4 - f.y1;
        float d2 = fabsf(((f.x2 - f.x4) * dy - (f.y2 - f.y4) * dx));
        float d3 = fabsf(((f.x3 - f.x4) * dy - (f.y3 - f.y4) * dx));
        float da1, da2;
        if (d2 >= 1.7f && d3 >= 1.7f) {
            if ((d2 + d3) * (d2 + d3) <= (dx * dx + dy * dy) * tol) {
                float a23 = pm_atan2f(f.y3 - f.y2, f.x3 - f.x2);
                da1       = fabsf(a23 - pm_atan2f(f.y2 - f.y1, f.x2 - f.x1));
                da2       = fabsf(pm_atan2f(f.y4 - f.y3, f.x4 - f.x3) - a23);
                if (da1 >= GB_PIF)
                    da1 = GB_2PIF - da1;
                if (da2 >= GB_PIF)
                    da2 = GB_2PIF - da2;
                if (da1 + da2 < 0.01f)
                    GB_EMIT1(s.x1234, s.y1234, GB_BEZ_MID)
                if (da1 > 0.01f)
                    GB_EMIT1(f.x2, f.y2, GB_BEZ_C2)
                if (da2 > 0.01f)
                    GB_EMIT1(f.x3, f.y3, GB_BEZ_C3)
            }
        } else {
            if (d2 >= 1.7f) {
                if (d2 * d2 <= tol * (dx * dx + dy * dy)) {
                    da1 = fabsf(pm_atan2f(f.y3 - f.y2, f.x3 - f.x2) - pm_atan2f(f.y2 - f.y1, f.x2 - f.x1));
                    if (da1 >= GB_PIF)
                        da1 = GB_2PIF - da1;
                    if (da1 <= 0.01f) {
                        s.n = 2, s.p0 = make_float2(f.x2, f.y2), s.p1 = make_float2(f.x3, f.y3);
                        s.w0 = GB_BEZ_C2, s.w1 = GB_BEZ_C3;
                        return;
                    }
                    if (da1 > 0.01f)
                        GB_EMIT1(f.x2, f.y2, GB_BEZ_C2)
                }
            } else if (d3 >= 1.7f) {
                if (d3 * d3 <= tol * (dx * dx + dy * dy)) {
                    da1 = fabsf(pm_atan2f(f.y4 - f.y3, f.x4 - f.x3) - pm_atan2f(f.y3 - f.y2, f.x3 - f.x2));
                    if (da1 >= GB_PIF)
                        da1 = GB_2PIF - da1;
                    if (da1 <= 0.01f) {
                        s.n = 2, s.p0 = make_float2(f.x2, f.y2), s.p1 = make_float2(f.x3, f.y3);
                        s.w0 = GB_BEZ_C2, s.w1 = GB_BEZ_C3;
                        return;
                    }
                    if (da1 > 0.01f)
                        GB_EMIT1(f.x3, f.y3, GB_BEZ_C3)
                }
            } else {
                float ex = s.x1234 - (f.x1 + f.x4) / 2;
                float ey = s.y1234 - (f.y1 + f.y4) / 2;
                if (ex * ex + ey * ey <= tol)
                    GB_EMIT1(s.x1234, s.y1234, GB_BEZ_MID)
            }
        }
    }
#undef GB_EMIT1
    s.sub = true;
}

/* Walk the subdivision tree of one cubic, calling emit(x, y, which, ta, tb)
   for every point _recursive_bezier would add.  Returns false if the node cap
   (cap nodes visited) was hit. */
template <bool TRACK, class Emit>
__device__ __forceinline__ bool gb_bezier_walk(float tol, float x1, float y1, float x2, float y2, float x3, float y3,
                                               float x4, float y4, Emit &emit, unsigned cap = GB_CURVE_NODE_CAP) {
    gb_bez_frame st[102];
    float2       tt[TRACK ? 102 : 1];
    int          sp = 0;
    if (TRACK)
        tt[0] = make_float2(0.f, 1.f);
    st[sp++]       = {x1, y1, x2, y2, x3, y3, x4, y4, 0u};
    unsigned nodes = 0;
    while (sp > 0) {
        --sp;
        gb_bez_frame f  = st[sp];
        float2       ti = TRACK ? tt[sp] : make_float2(0.f, 0.f);
        if (++nodes > cap)
            return false;
        if (f.level > 100u)
            continue;
        gb_bez_step s;
        gb_bez_eval(tol, f, s);
        if (!s.sub) {
            emit(s.p0.x, s.p0.y, s.w0, ti.x, ti.y);
            if (s.n == 2)
                emit(s.p1.x, s.p1.y, s.w1, ti.x, ti.y);
            continue;
        }
        /* subdivide: left half first, so push the right half below it */
        float tm = (ti.x + ti.y) * 0.5f;
        if (TRACK) {
            tt[sp]     = make_float2(tm, ti.y);
            tt[sp + 1] = make_float2(ti.x, tm);
        }
        st[sp++] = {s.x1234, s.y1234, s.x234, s.y234, s.x34, s.y34, f.x4, f.y4, f.level + 1u};
        st[sp++] = {f.x1, f.y1, s.x12, s.y12, s.x123, s.y123, s.x1234, s.y1234, f.level + 1u};
    }
    return true;
}

/* Weights of the four control points in an emitted point: the blossom of the
   sub-curve [ta, tb] at (ta,tb,tb)-style arguments.  MID = B(tm,tm,tm),
   C2 = B(ta,ta,tb), C3 = B(ta,tb,tb). */
__device__ __forceinline__ void gb_bez_weights(int which, float ta, float tb, float w[4]) {
    float u, v, s;
    if (which == GB_BEZ_MID) {
        u = v = s = (ta + tb) * 0.5f;
    } else if (which == GB_BEZ_C2) {
        u = ta, v = ta, s = tb;
    } else {
        u = ta, v = tb, s = tb;
    }
    float iu = 1.f - u, iv = 1.f - v, is = 1.f - s;
    w[0] = iu * iv * is;
    w[1] = u * iv * is + iu * v * is + iu * iv * s;
    w[2] = u * v * is + u * iv * s + iu * v * s;
    w[3] = u * v * s;
}

/* ---- the same tree, breadth first, by one warp ----
 *
 * Level by level, each lane evaluates one node of the level (gb_bez_eval:
 * the same operations, so the same decisions and the same points); children
 * and added points are compacted with warp ballots.  A node's key is its path
 * from the root, left-aligned (bit 63 - l set when the node is the right
 * half at level l + 1); a point's key is its node's, plus 1 for the second
 * point of a node that adds two.  Keys are distinct and sort the points in
 * depth-first order, which is _recursive_bezier's order.  A tree wider than
 * GB_BW_FCAP nodes at a level, with more than GB_BW_PCAP points, deeper than
 * 61 levels or with a NaN point returns -1: the caller walks it serially. */
#define GB_BW_FCAP 64
#define GB_BW_PCAP 96

struct gb_bw_node {
    gb_bez_frame       f;
    unsigned long long key;
};
struct gb_bw_pt {
    unsigned long long key;
    float2             p;
    int                which;
    unsigned           level;
};
struct gb_bw_smem {
    gb_bw_node fr[2][GB_BW_FCAP];
    gb_bw_pt   pt[GB_BW_PCAP];
};

/* all 32 lanes of the warp call this; returns the number of points in sm.pt */
__device__ __forceinline__ int gb_bezier_warp(float tol, float x1, float y1, float x2, float y2, float x3, float y3,
                                              float x4, float y4, gb_bw_smem &sm) {
    const unsigned lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
    if (lane == 0)
        sm.fr[0][0] = {{x1, y1, x2, y2, x3, y3, x4, y4, 0u}, 0ull};
    __syncwarp();
    int      nf = 1, cur = 0, npt = 0;
    unsigned nodes = 0;
    for (unsigned level = 0; nf > 0; level++) {
        nodes += (unsigned)nf;
        if (level > 61u || nodes > GB_CURVE_NODE_CAP)
            return -1;
        int nn = 0;
        for (int base = 0; base < nf; base += 32) {
            int         i   = base + (int)lane;
            bool        act = i < nf;
            gb_bw_node  nd;
            gb_bez_step s;
            s.sub = false, s.n = 0;
            if (act) {
                nd = sm.fr[cur][i];
                gb_bez_eval(tol, nd.f, s);
            }
            bool     nan  = act && !s.sub && ((s.p0.x != s.p0.x || s.p0.y != s.p0.y) ||
                                          (s.n == 2 && (s.p1.x != s.p1.x || s.p1.y != s.p1.y)));
            unsigned msub = __ballot_sync(0xffffffffu, act && s.sub);
            unsigned m1   = __ballot_sync(0xffffffffu, act && !s.sub && s.n >= 1);
            unsigned m2   = __ballot_sync(0xffffffffu, act && !s.sub && s.n == 2);
            if (__any_sync(0xffffffffu, nan))
                return -1;
            int csub = __popc(msub), cpt = __popc(m1) + __popc(m2);
            if (2 * (nn + csub) > GB_BW_FCAP || npt + cpt > GB_BW_PCAP)
                return -1;
            if (act && s.sub) {
                int                o   = 2 * (nn + __popc(msub & lt));
                unsigned long long bit = 1ull << (63u - level);
                sm.fr[cur ^ 1][o]      = {{nd.f.x1, nd.f.y1, s.x12, s.y12, s.x123, s.y123, s.x1234, s.y1234,
                                          level + 1u}, nd.key};
                sm.fr[cur ^ 1][o + 1]  = {{s.x1234, s.y1234, s.x234, s.y234, s.x34, s.y34, nd.f.x4, nd.f.y4,
                                          level + 1u}, nd.key | bit};
            }
            if (act && !s.sub && s.n) {
                int o      = npt + __popc(m1 & lt) + __popc(m2 & lt);
                sm.pt[o]   = {nd.key, s.p0, s.w0, level};
                if (s.n == 2)
                    sm.pt[o + 1] = {nd.key | 1ull, s.p1, s.w1, level};
            }
            nn += csub, npt += cpt;
        }
        __syncwarp();
        nf = 2 * nn, cur ^= 1;
    }
    return npt;
}

/* depth-first rank of point i among the warp's n points */
__device__ __forceinline__ int gb_bw_rank(const gb_bw_smem &sm, int n, int i) {
    unsigned long long k = sm.pt[i].key;
    int                r = 0;
    for (int j = 0; j < n; j++)
        r += sm.pt[j].key < k;
    return r;
}

/* the sub-curve interval of a point: its node's path as a dyadic interval */
__device__ __forceinline__ float2 gb_bw_interval(const gb_bw_pt &q) {
    float ta = __ull2float_rz(q.key & ~1ull) * 5.42101086242752217e-20f; /* 2^-64 */
    return make_float2(ta, ta + __int_as_float((127 - (int)q.level) << 23));
}
