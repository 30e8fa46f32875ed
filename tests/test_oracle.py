"""CPU checks of the oracle (no GPU): vkvg's own behavioural tests restated as
known-answer tests, agreement of the oracle's two raster modes, the committed
golden fixtures, an independent pure-Python flattening, and the size of the
portable-math substitution.  Also the product library's host-only matrix
functions against the same known answers."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle_bind as ob
import parity_util as pu
import pyref
from vkvg_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def ulp_eq(a, b, ulps=4):
    """gtest's EXPECT_FLOAT_EQ: within 4 units in the last place"""
    a, b = np.float32(a), np.float32(b)
    if a == b:
        return True
    ia, ib = int(a.view(np.int32)), int(b.view(np.int32))
    if (ia < 0) != (ib < 0):
        return False
    return abs(ia - ib) <= ulps


class Mat(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("xx", "yx", "xy", "yy", "x0", "y0")]


def check_mat(m, *want):
    got = (m.xx, m.yx, m.xy, m.yy, m.x0, m.y0)
    return all(ulp_eq(g, w) for g, w in zip(got, want))


def _matrix_libs():
    libs = [("oracle", ob.lib(), "vko_")]
    try:
        import vkvg_gb300

        vkvg_gb300._build.build()
        libs.append(("gb300", vkvg_gb300.lib(), "vkvg_"))
    except Exception as e:  # the product library must build here; report it
        pytest.fail("vkvg_gb300 library unavailable: %s" % e)
    return libs


def test_matrix_kat():
    """gunit_tests/matrices.cpp:10-70 (MatixInit, MatixIvert)"""
    cos2, sin2 = float(np.float32(np.cos(np.float32(2)))), float(np.float32(np.sin(np.float32(2))))
    for name, L, p in _matrix_libs():
        f = lambda n: getattr(L, p + n)
        for n, args in (("matrix_init", [C.c_float] * 6), ("matrix_init_translate", [C.c_float] * 2),
                        ("matrix_init_scale", [C.c_float] * 2), ("matrix_init_rotate", [C.c_float]),
                        ("matrix_get_scale", [C.POINTER(C.c_float)] * 2)):
            f(n).argtypes = [C.POINTER(Mat)] + args
        f("matrix_invert").restype = C.c_int
        m = Mat(1, 0, 0, 1, 0, 0)
        f("matrix_init_identity")(C.byref(m))
        assert check_mat(m, 1, 0, 0, 1, 0, 0), name
        f("matrix_init")(C.byref(m), 1.3, 2.5, 0.3, 0.7, 1.2, 1.7)
        assert check_mat(m, 1.3, 2.5, 0.3, 0.7, 1.2, 1.7), name
        f("matrix_init_translate")(C.byref(m), 1.3, 2.5)
        assert check_mat(m, 1, 0, 0, 1, 1.3, 2.5), name
        f("matrix_init_scale")(C.byref(m), 2.1, 1.5)
        assert check_mat(m, 2.1, 0, 0, 1.5, 0, 0), name
        a, b = C.c_float(), C.c_float()
        f("matrix_get_scale")(C.byref(m), C.byref(a), C.byref(b))
        assert ulp_eq(a.value, 2.1) and ulp_eq(b.value, 1.5), name
        f("matrix_init_rotate")(C.byref(m), 2.0)
        assert check_mat(m, cos2, sin2, -sin2, cos2, 0, 0), name
        # MatixIvert
        m = Mat(0, 0, 0, 0, 0, 0)
        assert f("matrix_invert")(C.byref(m)) == 5  # VKVG_STATUS_INVALID_MATRIX
        m = Mat(1, 1, 0, 0, 0, 0)
        assert f("matrix_invert")(C.byref(m)) == 5
        m = Mat(1, 0, 0, 1, 0, 0)
        assert f("matrix_invert")(C.byref(m)) == 0 and check_mat(m, 1, 0, 0, 1, 0, 0)
        f("matrix_init_scale")(C.byref(m), 2.1, 1.5)
        assert f("matrix_invert")(C.byref(m)) == 0
        assert check_mat(m, float(np.float32(1) / np.float32(2.1)), 0, 0, float(np.float32(1) / np.float32(1.5)), 0, 0)
        f("matrix_init_translate")(C.byref(m), 2.1, 1.5)
        assert f("matrix_invert")(C.byref(m)) == 0 and check_mat(m, 1, 0, 0, 1, -2.1, -1.5)
        f("matrix_init_rotate")(C.byref(m), 2.0)
        assert f("matrix_invert")(C.byref(m)) == 0 and check_mat(m, cos2, -sin2, sin2, cos2, 0, 0), name


def test_context_current_point_kat():
    """gunit_tests/context.cpp:175-218 (CtxBasicPathCommands) on the oracle"""
    surf = ob.OracleSurface(64, 64, 4)
    ctx = surf.context()

    def no_cp():
        return (not ctx.has_current_point()) and ctx.current_point() == (0.0, 0.0)

    assert no_cp()
    ctx.new_path()
    ctx.close_path()
    ctx.new_sub_path()
    assert no_cp()
    ctx.line_to(50, 10)
    assert ctx.current_point() == (50.0, 10.0)
    ctx.move_to(10, 50)
    assert ctx.has_current_point() and ctx.current_point() == (10.0, 50.0)
    ctx.line_to(50, 10)
    assert ctx.current_point() == (50.0, 10.0)
    ctx.rel_line_to(10, 10)
    assert ctx.current_point() == (60.0, 20.0)
    ctx.close_path()
    assert no_cp()
    ctx.line_to(50, 10)
    ctx.rel_line_to(10, 10)
    ctx.new_sub_path()
    assert no_cp()
    ctx.line_to(50, 10)
    ctx.rel_line_to(10, 10)
    ctx.new_path()
    assert no_cp()
    assert ctx.status() == 0
    ctx.destroy()
    surf.destroy()


def small_scenes():
    return [scenes.plain_small(n_polys=12, size=96, seed=0),
            scenes.curve_heavy(n_paths=10, size=128, seed=1, n_min=3, n_max=6),
            scenes.api_mix(n_items=24, size=160, seed=5),
            scenes.gradient_mix(n_items=14, size=144, seed=9),
            scenes.clip_mix(n_items=10, size=128, seed=13),
            scenes.gradient_mix(n_items=14, size=144, seed=9, radial=True),
            scenes.surface_mix(n_items=12, size=128, seed=23)]


@pytest.mark.parametrize("sc", small_scenes(), ids=lambda s: s["name"])
def test_literal_equals_scanline(sc):
    """the fan + stencil restatement and the crossing restatement give the same
    per-sample coverage for every draw and the same samples"""
    s0, c0 = pu.run_oracle(ob, sc, raster_mode=0)
    s1, c1 = pu.run_oracle(ob, sc, raster_mode=1)
    W, H, S = sc["width"], sc["height"], sc["samples"]
    draws = c0.draws()
    assert len(draws) == len(c1.draws())
    for i, d in enumerate(draws):
        if d["kind"] in (0, 1, 2, 5, 6):
            ob.lib().vko_set_raster_mode(0)
            a = c0.coverage(i, W, H, S)
            ob.lib().vko_set_raster_mode(1)
            b = c0.coverage(i, W, H, S)
            assert np.array_equal(a, b), (sc["name"], i, d["kind"])
    ob.lib().vko_set_raster_mode(0)
    assert np.array_equal(s0.samples_rgba(), s1.samples_rgba())
    assert np.array_equal(s0.image(), s1.image())


def sys_path_golden():
    import sys

    if GOLDEN not in sys.path:
        sys.path.insert(0, GOLDEN)


def _golden_path(name):
    return os.path.join(GOLDEN, name + ".npz")


@pytest.mark.parametrize("sc", small_scenes(), ids=lambda s: s["name"])
def test_oracle_matches_golden(sc):
    """the oracle against its committed outputs (tests/golden/make_golden.py)"""
    sys_path_golden()
    import make_golden

    g = np.load(_golden_path(sc["name"]))
    cur = make_golden.capture(sc)
    assert sorted(g.files) == sorted(cur.keys())
    for k in g.files:
        assert np.array_equal(g[k], cur[k]), (sc["name"], k)


def _atan2f(y, x):
    return ob.pmath(0, np.array([y], np.float32), np.array([x], np.float32))[0]


@pytest.mark.parametrize("scale", [1.0, 2.0])
def test_flattening_matches_python_restatement(scale):
    r = scenes.SplitMix64(11)
    for case in range(40):
        p0 = (r.rnd() * 200, r.rnd() * 200)
        cubics = [tuple(r.rnd() * 200 for _ in range(6)) for _ in range(1 + case % 4)]
        if case % 7 == 3:  # nearly collinear control points
            x0, y0 = p0
            cubics = [(x0 + 10, y0 + 10.001, x0 + 20, y0 + 19.999, x0 + 30, y0 + 30)]
        want = pyref.flatten_path(p0, cubics, _atan2f, scale)
        surf = ob.OracleSurface(256, 256, 4)
        ctx = surf.context()
        ctx.keep_draws(1)
        if scale != 1.0:
            ctx.scale(scale, scale)
        ctx.move_to(*p0)
        for c in cubics:
            ctx.curve_to(*c)
        ctx.fill()
        ctx.flush()
        d = [d for d in ctx.draws() if d["kind"] in (0, 1)]
        assert len(d) == 1
        got = d[0]["points"]
        assert got.shape == want.shape, (case, got.shape, want.shape)
        assert np.array_equal(got, want), case
        ctx.destroy()
        surf.destroy()


def test_portable_math_vs_libm():
    """vkvg calls the C library's atan2f/acosf/cosf/sinf; the oracle and the
    kernels use one portable implementation so host and device agree bit for
    bit.  Measure what the substitution changes on a curve-and-stroke scene
    and require it to stay inside the drop-in's image tolerance
    (<= 1/255 on 99.9 % of pixel channels, <= 2/255 everywhere)."""
    sc = scenes.curve_heavy(n_paths=24, size=192, seed=1, n_min=3, n_max=8)
    L = ob.lib()
    try:
        L.vko_set_math_mode(0)
        s0, _ = pu.run_oracle(ob, sc)
        L.vko_set_math_mode(1)
        s1, _ = pu.run_oracle(ob, sc)
    finally:
        L.vko_set_math_mode(0)
    a, b = s0.image().astype(np.int32), s1.image().astype(np.int32)
    diff = np.abs(a - b)
    assert (diff <= 1).mean() >= 0.999, (diff > 1).mean()
    assert diff.max() <= 2, diff.max()


def _np_smoothstep(e0, e1, x):
    f = np.float32
    t = (x - f(e0)) / (f(e1) - f(e0))
    t = np.minimum(np.maximum(t, f(0)), f(1))
    return (t * t) * (f(3) - f(2) * t)


def _np_mix(x, y, a):
    f = np.float32
    return x * (f(1) - a) + y * a


def test_linear_gradient_kat():
    """a gradient painted on a cleared surface equals an independent numpy
    fp32 evaluation of vkvg's LINEAR fragment expression
    (shaders/vkvg_main.frag:83-108): horizontal and diagonal axes, three stops"""
    f = np.float32
    W, H = 64, 24
    for (x0, y0, x1, y1) in ((8.0, 0.0, 56.0, 0.0), (60.0, 2.0, 4.0, 20.0)):
        stops = [(0.0, 1.0, 0.0, 0.0, 1.0), (0.4, 0.0, 1.0, 0.0, 0.5), (1.0, 0.0, 0.0, 1.0, 1.0)]
        surf = ob.OracleSurface(W, H, 4)
        ctx = surf.context()
        ctx.set_source_linear(x0, y0, x1, y1, stops)
        ctx.paint()
        ctx.flush()
        got = surf.premult()
        ctx.destroy()
        surf.destroy()
        px = np.arange(W, dtype=f)[None, :].repeat(H, 0)
        py = np.arange(H, dtype=f)[:, None].repeat(W, 1)
        p_x, p_y = (px + f(0.5)) / f(W), (py + f(0.5)) / f(H)
        p0x, p0y, p1x, p1y = f(x0) / f(W), f(y0) / f(H), f(x1) / f(W), f(y1) / f(H)
        dx, dy = p1x - p0x, p1y - p0y
        l = np.sqrt(dx * dx + dy * dy)
        ux, uy = dx / l, dy / l
        if uy == 0:
            dist = (p_x - p0x) / l
            dist = -dist if ux < 0 else dist
        else:
            m = -ux / uy
            bb = p0y - m * p0x
            dist = ((p_y - m * p_x - bb) / np.sqrt(f(1) + m * m)) / l
            dist = -dist if uy < 0 else dist
        cols = [np.array([a * r, a * g, a * b, a], f) for (_, r, g, b, a) in stops]
        t = _np_smoothstep(stops[0][0], stops[1][0], dist)
        c = [_np_mix(cols[0][k], cols[1][k], t) for k in range(4)]
        for i in range(1, len(stops) - 1):
            t = _np_smoothstep(stops[i][0], stops[i + 1][0], dist)
            c = [_np_mix(c[k], cols[i + 1][k], t) for k in range(4)]
        want = np.stack([np.rint(np.clip(ck * f(255), 0, 255)).astype(np.uint8) for ck in c], -1)
        assert np.array_equal(got, want)


def test_radial_gradient_kat():
    """a radial gradient painted on a cleared surface equals an independent
    numpy fp32 evaluation of vkvg's RADIAL fragment expression
    (shaders/vkvg_main.frag:109-144) after vkvg_pattern_edit_radial's focus
    adjustment (src/vkvg_pattern.c:95-119): a focus inside the outer circle,
    and one that edit_radial pulls inside"""
    f = np.float32
    W, H = 48, 40
    stops = [(0.0, 1.0, 1.0, 0.0, 1.0), (0.5, 0.0, 0.5, 1.0, 0.8), (1.0, 0.2, 0.0, 0.4, 1.0)]
    for (cx0, cy0, r0, cx1, cy1, r1) in ((20.0, 18.0, 3.0, 24.0, 20.0, 30.0), (40.0, 5.0, 2.0, 22.0, 20.0, 16.0)):
        surf = ob.OracleSurface(W, H, 4)
        ctx = surf.context()
        ctx.set_source_radial(cx0, cy0, r0, cx1, cy1, r1, stops)
        ctx.paint()
        ctx.flush()
        got = surf.premult()
        ctx.destroy()
        surf.destroy()
        # edit_radial
        r0, r1 = f(r0), f(r1)
        if r0 > r1 - f(1):
            r0 = r1 - f(1)
        ux, uy = f(cx0) - f(cx1), f(cy0) - f(cy1)
        l = np.sqrt(ux * ux + uy * uy)
        c0x, c0y = f(cx0), f(cy0)
        if l + r0 + f(1) >= r1:
            k = r1 - r0 - f(1)
            c0x, c0y = f(cx1) + (ux / l) * k, f(cy1) + (uy / l) * k
        # fragment stage, per pixel centre
        px = np.arange(W, dtype=f)[None, :].repeat(H, 0)
        py = np.arange(H, dtype=f)[:, None].repeat(W, 1)
        p_x, p_y = (px + f(0.5)) / f(W), (py + f(0.5)) / f(H)
        a0x, a0y, a1x, a1y = c0x / f(W), c0y / f(H), f(cx1) / f(W), f(cy1) / f(H)
        q0, q1 = r0 / f(W), r1 / f(W)
        dfx, dfy = a0x - a1x, a0y - a1y
        vx, vy = p_x - a0x, p_y - a0y
        vlen = np.sqrt(vx * vx + vy * vy)
        rx, ry = vx / vlen, vy / vlen
        a = rx * rx + ry * ry
        b = f(2) * (rx * dfx + ry * dfy)
        cc = (dfx * dfx + dfy * dfy) - q1 * q1
        disc = b * b - f(4) * a * cc
        with np.errstate(invalid="ignore"):
            t = (-b + np.sqrt(np.abs(disc))) / (f(2) * a)
            qx, qy = (a0x + rx * t) - a0x, (a0y + ry * t) - a0y
            glen = np.where(disc >= 0, np.sqrt(qx * qx + qy * qy) - q0, f(1)).astype(f)
        grad = (vlen - q0) / glen
        cols = [np.array([al * r, al * g, al * bb, al], f) for (_, r, g, bb, al) in stops]
        tt = _np_smoothstep(stops[0][0], stops[1][0], grad)
        c = [_np_mix(cols[0][k], cols[1][k], tt) for k in range(4)]
        for i in range(2, len(stops)):
            tt = _np_smoothstep(stops[i - 1][0], stops[i][0], grad)
            c = [_np_mix(c[k], cols[i][k], tt) for k in range(4)]
        want = np.stack([np.rint(np.clip(np.nan_to_num(ck * f(255), nan=0.0), 0, 255)).astype(np.uint8)
                         for ck in c], -1)
        assert np.array_equal(got, want)


def _np_wrap(i, n, extend):
    if extend == 1:
        return i % n
    if extend == 2:
        t = (i % (2 * n)) - n
        return (n - 1) - np.where(t >= 0, t, -(1 + t))
    if extend == 3:
        return np.clip(i, 0, n - 1)
    return np.where((i < 0) | (i >= n), -1, i)


def test_surface_source_kat():
    """a 5x3 source of solid pixels painted through a surface pattern equals
    an independent numpy evaluation of the SURFACE fragment case
    (shaders/vkvg_main.frag:72-82) and Vulkan's texel filtering: nearest and
    bilinear (8-bit weights), each extend mode, a pattern matrix"""
    f = np.float32
    rng = np.random.default_rng(3)
    sw, sh = 5, 3
    cols = rng.integers(0, 256, (sh, sw, 3))
    W, H = 40, 28
    for extend in range(4):
        for filt, bil in ((3, False), (4, True)):  # VKVG_FILTER_NEAREST, _BILINEAR
            src = ob.OracleSurface(sw, sh, 4)
            c = src.context()
            for y in range(sh):
                for x in range(sw):
                    r, g, b = cols[y, x] / 255.0
                    c.set_source_rgb(float(r), float(g), float(b))
                    c.rectangle(float(x), float(y), 1.0, 1.0)
                    c.fill()
            c.flush()
            c.destroy()
            texels = src.premult()
            pm = (0.37, 0.05, -0.08, 0.29, 1.3, -0.7)  # pattern matrix, folded into the inverse matrix
            dst = ob.OracleSurface(W, H, 4)
            c = dst.context()
            c.set_source_surface_pattern(src, extend, filt, pm)
            c.paint()
            c.flush()
            got = dst.premult()
            c.destroy()
            px = np.arange(W, dtype=f)[None, :].repeat(H, 0) + f(0.5)
            py = np.arange(H, dtype=f)[:, None].repeat(W, 1) + f(0.5)
            xx, yx, xy, yy, x0, y0 = [f(v) for v in pm]
            u = (xx * px + xy * py + x0) / f(sw)
            v = (yx * px + yy * py + y0) / f(sh)
            us, vs = u * f(sw), v * f(sh)
            tex = texels.astype(f) / f(255)

            def fetch(i, j):
                i, j = _np_wrap(i, sw, extend), _np_wrap(j, sh, extend)
                ok = (i >= 0) & (j >= 0)
                return np.where(ok[..., None], tex[np.maximum(j, 0), np.maximum(i, 0)], f(0))

            if not bil:
                out = fetch(np.floor(us).astype(np.int64), np.floor(vs).astype(np.int64))
            else:
                a, b = us - f(0.5), vs - f(0.5)
                al = np.floor((a - np.floor(a)) * f(256)) * f(1 / 256)
                be = np.floor((b - np.floor(b)) * f(256)) * f(1 / 256)
                i, j = np.floor(a).astype(np.int64), np.floor(b).astype(np.int64)
                w = [((f(1) - al) * (f(1) - be))[..., None], (al * (f(1) - be))[..., None],
                     ((f(1) - al) * be)[..., None], (al * be)[..., None]]
                out = w[0] * fetch(i, j) + w[1] * fetch(i + 1, j)
                out = out + w[2] * fetch(i, j + 1)
                out = out + w[3] * fetch(i + 1, j + 1)
            want = np.rint(np.clip(out * f(255), 0, 255)).astype(np.uint8)
            assert np.array_equal(got, want), (extend, filt, int((got != want).sum()))
            dst.destroy()
            src.destroy()


def test_pattern_api_semantics():
    """vkvg's pattern object behaviour (src/vkvg_pattern.c) on both libraries:
    reference counts, stop count, type and the 16-stop limit"""
    import vkvg_gb300

    vkvg_gb300._build.build()
    for L, pre in ((ob.lib(), "vko_"), (vkvg_gb300.lib(), "vkvg_")):
        f = lambda n: getattr(L, pre + n)
        p = f("pattern_create_linear")(0.0, 0.0, 10.0, 0.0)
        assert f("pattern_status")(p) == 0
        assert f("pattern_get_reference_count")(p) == 1
        f("pattern_reference")(p)
        assert f("pattern_get_reference_count")(p) == 2
        for i in range(16):
            assert f("pattern_add_color_stop")(p, i / 15.0, 1.0, 0.5, 0.25, 0.5) == 0
        assert f("pattern_add_color_stop")(p, 1.0, 1.0, 1.0, 1.0, 1.0) == 7  # VKVG_STATUS_INVALID_INDEX
        n = C.c_uint32()
        assert f("pattern_get_color_stop_count")(p, C.byref(n)) == 0 and n.value == 16
        f("pattern_destroy")(p)
        assert f("pattern_get_reference_count")(p) == 1
        assert f("pattern_edit_radial")(p, 0.0, 0.0, 1.0, 0.0, 0.0, 9.0) == 9  # PATTERN_TYPE_MISMATCH
        f("pattern_destroy")(p)
        q = f("pattern_create_radial")(1.0, 2.0, 3.0, 4.0, 5.0, 20.0)
        assert f("pattern_status")(q) == 0 and f("pattern_get_reference_count")(q) == 1
        assert f("pattern_edit_linear")(q, 0.0, 0.0, 1.0, 1.0) == 9
        assert f("pattern_edit_radial")(q, 0.0, 0.0, 30.0, 1.0, 1.0, 10.0) == 0  # radius0 clamped, focus moved
        f("pattern_destroy")(q)
    L = vkvg_gb300.lib()
    q = L.vkvg_pattern_create_radial(0.0, 0.0, 1.0, 0.0, 0.0, 5.0)
    assert L.vkvg_pattern_get_type(q) == 3  # VKVG_PATTERN_TYPE_RADIAL
    L.vkvg_pattern_destroy(q)
    p = L.vkvg_pattern_create_linear(0.0, 0.0, 1.0, 1.0)
    assert L.vkvg_pattern_get_type(p) == 2  # VKVG_PATTERN_TYPE_LINEAR
    L.vkvg_pattern_add_color_stop(p, 0.0, 1.0, 0.5, 0.25, 0.5)
    o, r, g, b, a = (C.c_float() for _ in range(5))
    assert L.vkvg_pattern_get_color_stop_rgba(p, 0, C.byref(o), C.byref(r), C.byref(g), C.byref(b), C.byref(a)) == 0
    assert (r.value, g.value, b.value, a.value) == (0.5, 0.25, 0.125, 0.5)  # premultiplied, as vkvg stores them
    assert L.vkvg_pattern_get_color_stop_rgba(p, 1, C.byref(o), C.byref(r), C.byref(g), C.byref(b),
                                              C.byref(a)) == 7
    L.vkvg_pattern_destroy(p)


@pytest.mark.parametrize("sc", scenes.vkvg_clip_cases(width=256, height=200) +
                         [scenes.clip_mix(n_items=10, size=96, seed=3, samples=1, flush_every=3)],
                         ids=lambda s: s["name"])
def test_clip_literal_equals_scanline(sc):
    """clip scenes: the literal stencil passes and the crossing restatement
    give the same samples"""
    s0, c0 = pu.run_oracle(ob, sc, raster_mode=0)
    s1, c1 = pu.run_oracle(ob, sc, raster_mode=1)
    ob.lib().vko_set_raster_mode(0)
    assert c0.status() == 0 and c1.status() == 0
    assert np.array_equal(s0.samples_rgba(), s1.samples_rgba())


def _clip_row(ops, w=16, h=16):
    """green channel of row 8 after the ops on a fresh 16x16 surface, and the
    context status"""
    sc = {"name": "clip_kat", "width": w, "height": h, "samples": 4, "ops": ops, "paths": 0}
    s, c = pu.run_oracle(ob, sc)
    row = s.image()[8, :, 1]
    return "".join("#" if v > 200 else ("+" if v else ".") for v in row), c.status()


def test_clip_state_machine_kat():
    """vkvg's clip / save / restore behaviour (src/vkvg_context.c:698-795,
    1251-1512) on 16x16 cases, including two outcomes of its state machine
    that a reader might not expect: a restore finding curClipState "none"
    leaves the stencil alone (so two nested levels restore only one), and
    reset_clip clears the save bits of the levels below it"""
    R = lambda x0, x1: ("rectangle", float(x0), 2.0, float(x1 - x0), 12.0)
    paint = [("set_source_rgb", 0.0, 1.0, 0.0), ("paint",)]
    inner, outer = "..######........", "....########...."
    cases = [
        ([R(2, 8), ("clip",)] + paint, inner),
        ([("save",), R(2, 8), ("clip",), ("restore",)] + paint, "#" * 16),
        ([("save",), R(2, 8), ("clip",), ("save",), R(4, 12), ("clip",), ("restore",)] + paint, inner),
        ([("save",), R(2, 8), ("clip",), ("save",), R(4, 12), ("clip",), ("restore",), ("restore",)] + paint, inner),
        ([R(4, 12), ("clip",), ("save",), R(2, 8), ("clip",), ("restore",)] + paint, outer),
        ([R(2, 8), ("clip",), ("save",), ("reset_clip",), ("restore",)] + paint, "#" * 16),
        ([R(2, 8), ("clip",), ("reset_clip",)] + paint, "#" * 16),
        ([R(2, 8), ("clip",), ("clear",)] + paint, "#" * 16),
        ([R(2, 8), ("clip_preserve",), ("set_source_rgb", 0.0, 1.0, 0.0), ("fill",), ("set_source_rgb", 0.0, 0.5, 0.0),
          R(4, 12), ("fill",)], "..##++++........"),
    ]
    for ops, want in cases:
        got, st = _clip_row(ops)
        assert st == 0 and got == want, (ops, got)
    got, st = _clip_row([("restore",)] + paint)
    assert st == 3 and got == "." * 16  # VKVG_STATUS_INVALID_RESTORE; later calls do nothing


def test_save_restore_state_kat():
    """vkvg_restore brings back line width, dashes, operator, fill rule, matrix
    and source, and sets the line join to miter (the field vkvg_save never
    writes)"""
    surf = ob.OracleSurface(32, 32, 4)
    ctx = surf.context()
    ctx.set_line_width(3.0)
    ctx.set_line_join(1)
    ctx.set_fill_rule(0)
    ctx.save()
    ctx.set_line_width(7.0)
    ctx.set_fill_rule(1)
    ctx.translate(5.0, 5.0)
    ctx.restore()
    assert ctx.get_line_width() == 3.0 and ctx.get_line_join() == 0 and ctx.get_fill_rule() == 0
    m = Mat()
    ob.lib().vko_get_matrix.argtypes = [C.c_void_p, C.POINTER(Mat)]
    ob.lib().vko_get_matrix(ctx.h, C.byref(m))
    assert (m.x0, m.y0) == (0.0, 0.0)
    assert ctx.status() == 0
    ctx.destroy()
    surf.destroy()
