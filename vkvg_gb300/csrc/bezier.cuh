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

/* Walk the subdivision tree of one cubic, calling emit(x, y, which, ta, tb)
   for every point _recursive_bezier would add.  Returns false if the node cap
   was hit. */
template <bool TRACK, class Emit>
__device__ __forceinline__ bool gb_bezier_walk(float tol, float x1, float y1, float x2, float y2, float x3, float y3,
                                               float x4, float y4, Emit &emit) {
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
        if (++nodes > GB_CURVE_NODE_CAP)
            return false;
        if (f.level > 100u)
            continue;
        float x12   = (f.x1 + f.x2) / 2;
        float y12   = (f.y1 + f.y2) / 2;
        float x23   = (f.x2 + f.x3) / 2;
        float y23   = (f.y2 + f.y3) / 2;
        float x34   = (f.x3 + f.x4) / 2;
        float y34   = (f.y3 + f.y4) / 2;
        float x123  = (x12 + x23) / 2;
        float y123  = (y12 + y23) / 2;
        float x234  = (x23 + x34) / 2;
        float y234  = (y23 + y34) / 2;
        float x1234 = (x123 + x234) / 2;
        float y1234 = (y123 + y234) / 2;
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
                    if (da1 + da2 < 0.01f) {
                        emit(x1234, y1234, GB_BEZ_MID, ti.x, ti.y);
                        continue;
                    }
                    if (da1 > 0.01f) {
                        emit(f.x2, f.y2, GB_BEZ_C2, ti.x, ti.y);
                        continue;
                    }
                    if (da2 > 0.01f) {
                        emit(f.x3, f.y3, GB_BEZ_C3, ti.x, ti.y);
                        continue;
                    }
                }
            } else {
                if (d2 >= 1.7f) {
                    if (d2 * d2 <= tol * (dx * dx + dy * dy)) {
                        da1 = fabsf(pm_atan2f(f.y3 - f.y2, f.x3 - f.x2) - pm_atan2f(f.y2 - f.y1, f.x2 - f.x1));
                        if (da1 >= GB_PIF)
                            da1 = GB_2PIF - da1;
                        if (da1 <= 0.01f) {
                            emit(f.x2, f.y2, GB_BEZ_C2, ti.x, ti.y);
                            emit(f.x3, f.y3, GB_BEZ_C3, ti.x, ti.y);
                            continue;
                        }
                        if (da1 > 0.01f) {
                            emit(f.x2, f.y2, GB_BEZ_C2, ti.x, ti.y);
                            continue;
                        }
                    }
                } else if (d3 >= 1.7f) {
                    if (d3 * d3 <= tol * (dx * dx + dy * dy)) {
                        da1 = fabsf(pm_atan2f(f.y4 - f.y3, f.x4 - f.x3) - pm_atan2f(f.y3 - f.y2, f.x3 - f.x2));
                        if (da1 >= GB_PIF)
                            da1 = GB_2PIF - da1;
                        if (da1 <= 0.01f) {
                            emit(f.x2, f.y2, GB_BEZ_C2, ti.x, ti.y);
                            emit(f.x3, f.y3, GB_BEZ_C3, ti.x, ti.y);
                            continue;
                        }
                        if (da1 > 0.01f) {
                            emit(f.x3, f.y3, GB_BEZ_C3, ti.x, ti.y);
                            continue;
                        }
                    }
                } else {
                    float ex = x1234 - (f.x1 + f.x4) / 2;
                    float ey = y1234 - (f.y1 + f.y4) / 2;
                    if (ex * ex + ey * ey <= tol) {
                        emit(x1234, y1234, GB_BEZ_MID, ti.x, ti.y);
                        continue;
                    }
                }
            }
        }
        /* subdivide: left half first, so push the right half below it */
        float tm = (ti.x + ti.y) * 0.5f;
        if (TRACK) {
            tt[sp]     = make_float2(tm, ti.y);
            tt[sp + 1] = make_float2(ti.x, tm);
        }
        st[sp++] = {x1234, y1234, x234, y234, x34, y34, f.x4, f.y4, f.level + 1u};
        st[sp++] = {f.x1, f.y1, x12, y12, x123, y123, x1234, y1234, f.level + 1u};
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
