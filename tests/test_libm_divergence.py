"""What vkvg's own libm arithmetic changes (CPU, no GPU).

vkvg calls the C library's atan2f, acosf, cosf and sinf in its branch
decisions: the angle tests of _recursive_bezier
(src/vkvg_context_internal.c:1360-1385), the join angle and round-join fan
of _build_vb_step (:961-967, :1100-1135) and the caps.  The GPU kernels and
the oracle share one portable implementation instead, so that host and device
agree bit for bit; the GPU is bit-exact against the oracle in that mode.
Here the oracle runs the benchmark's two single-surface configurations in
both math modes (portable, and this host's glibc as vkvg would call it) and
measures the difference at every stage:

* cubics whose subdivision differs (point count or points);
* draws whose vertex counts differ, and the largest vertex difference on
  draws with equal counts (the vertex bar, 1e-3 px);
* per-sample winding / covering counts of the draws whose geometry differs;
* the final samples and image (bar: within 1/255 on 99.9 % of channels and
  within 2/255 everywhere).

The measured figures (x86-64 glibc) are asserted as upper bounds, so that a
change of either implementation that widens the gap shows up."""
import os

import numpy as np
import pytest

import oracle_bind as ob
import parity_util as pu
from vkvg_gb300 import scenes


def _cubics(sc):
    """(p0, c1, c2, p3) of every curve_to of a scene, from its current point"""
    cur, out = None, []
    for op in sc["ops"]:
        if op[0] in ("move_to", "line_to"):
            cur = op[1:3]
        elif op[0] == "curve_to":
            out.append(cur + op[1:7])
            cur = op[5:7]
    return np.array(out, np.float32).reshape(-1, 8)


def _flatten_all(cubics, mode):
    L = ob.lib()
    L.vko_set_math_mode(mode)
    buf = np.zeros(2 * 8192, np.float32)
    out = []
    try:
        for c in cubics:
            c = np.ascontiguousarray(c)
            n = L.vko_flatten_cubic(np.float32(0.25), ob.ptr(c), ob.ptr(buf), 8192)
            out.append(buf[:2 * min(n, 8192)].copy())
    finally:
        L.vko_set_math_mode(0)
    return out


def _run(sc, mode):
    L = ob.lib()
    L.vko_set_math_mode(mode)
    try:
        return pu.run_oracle(ob, sc, threads=os.cpu_count() or 1)
    finally:
        L.vko_set_math_mode(0)


def _geometry_differs(x, y):
    if x["kind"] in (0, 1):
        return not np.array_equal(x["subpaths"], y["subpaths"]) or not np.array_equal(x["points"], y["points"])
    if x["kind"] == 2:
        return (x["verts"].shape != y["verts"].shape or not np.array_equal(x["inds"], y["inds"]) or
                not np.array_equal(x["verts"], y["verts"]))
    return False


def _measure(sc, coverage_draws=None):
    """every figure of the comparison for one scene"""
    m = {}
    cb = _cubics(sc)
    if len(cb):
        a, b = _flatten_all(cb, 0), _flatten_all(cb, 1)
        m["cubics"] = len(cb)
        m["cubics_diverging"] = sum(len(x) != len(y) or not np.array_equal(x, y) for x, y in zip(a, b))
    s0, c0 = _run(sc, 0)
    s1, c1 = _run(sc, 1)
    d0, d1 = c0.draws(), c1.draws()
    assert len(d0) == len(d1)
    m["draws"] = len(d0)
    count_diff, vmax, over = 0, 0.0, 0
    diff = []
    for i, (x, y) in enumerate(zip(d0, d1)):
        if not _geometry_differs(x, y):
            continue
        diff.append(i)
        if x["kind"] in (0, 1):
            same = np.array_equal(x["subpaths"], y["subpaths"])
            px, py = x["points"], y["points"]
        else:
            same = x["verts"].shape == y["verts"].shape and np.array_equal(x["inds"], y["inds"])
            px, py = x.get("verts"), y.get("verts")
        if not same:
            count_diff += 1
        elif len(px):
            dv = np.abs(px.astype(np.float64) - py).max(axis=1)
            vmax = max(vmax, float(dv.max()))
            over += int((dv > 1e-3).sum())
    m["draws_geometry_differs"] = len(diff)
    m["draws_count_differs"] = count_diff
    m["max_vertex_delta_equal_counts"] = vmax
    m["vertices_over_1e-3"] = over
    W, H, S = sc["width"], sc["height"], sc["samples"]
    bad, nbad = 0, 0
    L = ob.lib()
    for i in diff if coverage_draws is None else diff[:coverage_draws]:
        L.vko_set_math_mode(0)
        a = c0.coverage(i, W, H, S)
        L.vko_set_math_mode(1)
        b = c1.coverage(i, W, H, S)
        L.vko_set_math_mode(0)
        k = int((a != b).sum())
        bad += k
        nbad += k > 0
    m["draws_winding_differs"] = nbad
    m["samples_winding_differs"] = bad
    m["sample_draw_pairs"] = len(d0) * W * H * S
    ia, ib = s0.image().astype(np.int32), s1.image().astype(np.int32)
    d = np.abs(ia - ib)
    m["image_channels_over_1"] = float((d > 1).mean())
    m["image_max_delta"] = int(d.max())
    m["samples_differ"] = float((s0.samples_rgba() != s1.samples_rgba()).any(-1).mean())
    for o in (c0, c1):
        o.destroy()
    for s in (s0, s1):
        s.destroy()
    return m


def test_libm_divergence_small_polygons():
    """512x512, 64 self-intersecting polygons, NON_ZERO fill and a black
    width-4 miter stroke (seed 0).  Measured: no cubics; 49 of 129 draws
    (strokes) have vertices that differ, none in count; the largest vertex
    difference is 1.28e-3 px (the only vertex above 1e-3), on a sharp miter
    join where lh = hw / cos(a/2) amplifies one ulp of cosf; 5 of 135 M
    sample-draw windings differ (one stroke draw); the samples and the image
    are identical."""
    m = _measure(scenes.plain_small())
    assert m["draws_count_differs"] == 0, m
    assert m["max_vertex_delta_equal_counts"] < 2e-3 and m["vertices_over_1e-3"] <= 2, m
    assert m["samples_winding_differs"] <= 16, m
    assert m["image_channels_over_1"] <= 1e-3 and m["image_max_delta"] <= 2, m


@pytest.mark.timeout(600)
def test_libm_divergence_curve_heavy():
    """1024x1024, 2,048 closed paths of 4-64 cubics, both fill rules, every
    join and cap, dashes (seed 1).  Measured: 5 of 69,330 cubics subdivide
    differently; 145 of 4,097 draws have a different vertex count (mostly
    round joins and caps whose fan step count follows acosf); the largest
    vertex difference on draws of equal counts is 2.4e-4 px; windings are
    compared on the first 160 of the 1,588 draws whose geometry differs (no
    difference there; over all 1,588, measured once, 54 samples in 13 draws
    differ, of 17.2 G sample-draw pairs); the samples and the image are
    identical."""
    m = _measure(scenes.curve_heavy(), coverage_draws=160)
    assert m["cubics_diverging"] <= 20, m
    assert m["draws_count_differs"] <= 300, m
    assert m["max_vertex_delta_equal_counts"] < 1e-3, m
    assert m["samples_winding_differs"] / m["sample_draw_pairs"] < 1e-7, m
    assert m["image_channels_over_1"] <= 1e-3 and m["image_max_delta"] <= 2, m
