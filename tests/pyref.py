"""Independent pure-Python restatement of vkvg's cubic flattening, for small
cross-checks of the oracle (test infrastructure only).

Follows _curve_to (src/vkvg_context.c:541-566) and _recursive_bezier
(src/vkvg_context_internal.c:1305-1461) of vkvg line by line with numpy
float32 scalars, so every float operation rounds to fp32 as in C.  Where the C
code compares a float with a double constant (d2 > CURVE_COLLINEARITY_EPSILON,
da1 > M_CUSP_LIMIT, da1 < M_ANGLE_TOLERANCE) the comparison is made in double,
as C's usual arithmetic conversions do; where it casts the constant to float
((float)M_ANGLE_TOLERANCE) it is made in fp32.  M_2_PIF is vkvg's 2/pi
constant (src/vkvg_internal.h:45), which _recursive_bezier uses where 2*pi
would be expected; the restatement keeps it.  atan2f is passed in (the
portable implementation both the oracle and the kernels use).
"""
import numpy as np

F = np.float32
M_PIF = F(3.14159265358979323846)
M_2_PIF = F(0.63661977236758134308)
COLLINEARITY_EPS = 1.7
CUSP_LIMIT = 0.01
ANGLE_TOL = 0.01
RECURSION_LIMIT = 100


def recursive_bezier(out, tol, x1, y1, x2, y2, x3, y3, x4, y4, level, atan2f):
    if level > RECURSION_LIMIT:
        return
    two = F(2)
    x12, y12 = (x1 + x2) / two, (y1 + y2) / two
    x23, y23 = (x2 + x3) / two, (y2 + y3) / two
    x34, y34 = (x3 + x4) / two, (y3 + y4) / two
    x123, y123 = (x12 + x23) / two, (y12 + y23) / two
    x234, y234 = (x23 + x34) / two, (y23 + y34) / two
    x1234, y1234 = (x123 + x234) / two, (y123 + y234) / two
    if level > 0:
        dx, dy = x4 - x1, y4 - y1
        d2 = abs((x2 - x4) * dy - (y2 - y4) * dx)
        d3 = abs((x3 - x4) * dy - (y3 - y4) * dx)
        if float(d2) > COLLINEARITY_EPS and float(d3) > COLLINEARITY_EPS:
            if (d2 + d3) * (d2 + d3) <= (dx * dx + dy * dy) * tol:
                a23 = atan2f(y3 - y2, x3 - x2)
                da1 = abs(a23 - atan2f(y2 - y1, x2 - x1))
                da2 = abs(atan2f(y4 - y3, x4 - x3) - a23)
                if da1 >= M_PIF:
                    da1 = M_2_PIF - da1
                if da2 >= M_PIF:
                    da2 = M_2_PIF - da2
                if da1 + da2 < F(ANGLE_TOL):
                    out.append((x1234, y1234))
                    return
                if float(da1) > CUSP_LIMIT:
                    out.append((x2, y2))
                    return
                if float(da2) > CUSP_LIMIT:
                    out.append((x3, y3))
                    return
        elif float(d2) > COLLINEARITY_EPS:
            if d2 * d2 <= tol * (dx * dx + dy * dy):
                da1 = abs(atan2f(y3 - y2, x3 - x2) - atan2f(y2 - y1, x2 - x1))
                if da1 >= M_PIF:
                    da1 = M_2_PIF - da1
                if float(da1) < ANGLE_TOL:
                    out.append((x2, y2))
                    out.append((x3, y3))
                    return
                if float(da1) > CUSP_LIMIT:
                    out.append((x2, y2))
                    return
        elif float(d3) > COLLINEARITY_EPS:
            if d3 * d3 <= tol * (dx * dx + dy * dy):
                da1 = abs(atan2f(y4 - y3, x4 - x3) - atan2f(y3 - y2, x3 - x2))
                if da1 >= M_PIF:
                    da1 = M_2_PIF - da1
                if float(da1) < ANGLE_TOL:
                    out.append((x2, y2))
                    out.append((x3, y3))
                    return
                if float(da1) > CUSP_LIMIT:
                    out.append((x3, y3))
                    return
        else:
            dx = x1234 - (x1 + x4) / two
            dy = y1234 - (y1 + y4) / two
            if dx * dx + dy * dy <= tol:
                out.append((x1234, y1234))
                return
    recursive_bezier(out, tol, x1, y1, x12, y12, x123, y123, x1234, y1234, level + 1, atan2f)
    recursive_bezier(out, tol, x1234, y1234, x234, y234, x34, y34, x4, y4, level + 1, atan2f)


def flatten_path(p0, cubics, atan2f, scale=1.0):
    """points of move_to(p0) then curve_to(c) for each (x1, y1, x2, y2, x3, y3)
    in cubics, with a CTM of uniform scale `scale` (distance tolerance
    0.25 / scale, src/vkvg_context.c:556-558)"""
    tol = F(abs(F(0.25) / F(scale)))
    pts = [(F(p0[0]), F(p0[1]))]
    for c in cubics:
        x1, y1, x2, y2, x3, y3 = [F(v) for v in c]
        cx, cy = pts[-1]
        recursive_bezier(pts, tol, cx, cy, x1, y1, x2, y2, x3, y3, 0, atan2f)
        pts.append((x3, y3))
    return np.array(pts, np.float32)
