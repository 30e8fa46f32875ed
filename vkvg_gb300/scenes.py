"""Seeded synthetic scenes for the vkvg path hot path (benchmarks and tests).

A scene is a list of API calls ``(name, *args)`` that is replayed, call for
call, on any object exposing vkvg's context methods (the GPU library's Python
binding, or the CPU oracle).  Randomness comes from one splitmix64 stream per
scene; ``rnd()`` returns (x >> 40) * 2**-24, a float in [0, 1) that is exactly
representable in fp32, so the same scene is produced in C or Python.

Scenes (sizes follow the benchmark configurations; no public dataset exists
for this path, so seeded synthetic inputs stand in for real content):

* ``plain_small`` - 512x512 RGBA8, MSAA 4, white background, 64 closed
  polygons with n ~ U{3..32} vertices uniform in [0,512)^2 (self-intersecting
  allowed), seed 0.  Each is filled NON_ZERO in an opaque U[0,1) RGB colour,
  then stroked black at width 4, miter join (limit 10), butt cap.
* ``curve_heavy`` - 1024x1024, MSAA 4, white background, 2048 closed paths of
  n ~ U{4..64} cubic Beziers, control points uniform in [0,1024)^2, seed 1.
  Path i is filled EVEN_ODD when i is even and NON_ZERO when odd, colour RGB
  U[0,1) with alpha U[0.3,1); then stroked in a second such colour at width
  U[1,8), join i mod 3 (miter/round/bevel), cap i mod 3 (butt/round/square),
  dash [10, 5] offset 0 when i mod 4 == 0.
* ``api_mix`` - small surface exercising the rest of the path API: arcs in
  both directions, elliptic arcs (all flag combinations), ellipses,
  rectangles and rounded rectangles, quadratic and relative commands, sub
  paths, transforms, opacity, every join and cap, multi-entry dash patterns
  with offsets, and the CLEAR / DIFFERENCE operators.
* ``gradient_mix`` - linear gradient sources: horizontal, vertical, diagonal
  and reversed axes, 2 to 5 stops, opacity, pattern matrices and CTMs, a
  gradient paint, gradient strokes, and more distinct gradients than one
  frame holds.
"""

MASK64 = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed):
        self.s = seed & MASK64

    def next(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & MASK64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def rnd(self):
        return (self.next() >> 40) * (1.0 / 16777216.0)

    def randint(self, lo, hi):
        """uniform integer in [lo, hi]"""
        return lo + int(self.rnd() * (hi - lo + 1))


def plain_small(n_polys=64, size=512, seed=0):
    r = SplitMix64(seed)
    ops = [("set_source_rgb", 1.0, 1.0, 1.0), ("paint",)]
    ops += [("set_line_width", 4.0), ("set_line_join", 0), ("set_line_cap", 0), ("set_miter_limit", 10.0),
            ("set_fill_rule", 1)]
    for _ in range(n_polys):
        n = r.randint(3, 32)
        pts = [(r.rnd() * size, r.rnd() * size) for _ in range(n)]
        col = (r.rnd(), r.rnd(), r.rnd())
        ops.append(("move_to",) + pts[0])
        for p in pts[1:]:
            ops.append(("line_to",) + p)
        ops.append(("close_path",))
        ops.append(("set_source_rgb",) + col)
        ops.append(("fill_preserve",))
        ops.append(("set_source_rgb", 0.0, 0.0, 0.0))
        ops.append(("stroke",))
    return {"name": "plain_small", "width": size, "height": size, "samples": 4, "ops": ops, "paths": n_polys}


def curve_heavy(n_paths=2048, size=1024, seed=1, n_min=4, n_max=64):
    r = SplitMix64(seed)
    ops = [("set_source_rgb", 1.0, 1.0, 1.0), ("paint",), ("set_miter_limit", 10.0)]
    for i in range(n_paths):
        n = r.randint(n_min, n_max)
        p0 = (r.rnd() * size, r.rnd() * size)
        fill = (r.rnd(), r.rnd(), r.rnd(), 0.3 + 0.7 * r.rnd())
        stroke = (r.rnd(), r.rnd(), r.rnd(), 0.3 + 0.7 * r.rnd())
        width = 1.0 + 7.0 * r.rnd()
        ops.append(("move_to",) + p0)
        for k in range(n):
            c1 = (r.rnd() * size, r.rnd() * size)
            c2 = (r.rnd() * size, r.rnd() * size)
            end = p0 if k == n - 1 else (r.rnd() * size, r.rnd() * size)
            ops.append(("curve_to",) + c1 + c2 + end)
        ops.append(("close_path",))
        ops.append(("set_fill_rule", 0 if i % 2 == 0 else 1))
        ops.append(("set_source_rgba",) + fill)
        ops.append(("fill_preserve",))
        ops.append(("set_line_width", width))
        ops.append(("set_line_join", i % 3))
        ops.append(("set_line_cap", i % 3))
        ops.append(("set_dash", [10.0, 5.0] if i % 4 == 0 else [], 0.0))
        ops.append(("set_source_rgba",) + stroke)
        ops.append(("stroke",))
    return {"name": "curve_heavy", "width": size, "height": size, "samples": 4, "ops": ops, "paths": n_paths}


def api_mix(n_items=24, size=160, seed=5, samples=4):
    r = SplitMix64(seed)
    u = lambda lo, hi: lo + (hi - lo) * r.rnd()
    ops = [("set_source_rgb", 1.0, 1.0, 1.0), ("paint",)]
    for i in range(n_items):
        k = i % 8
        ops.append(("identity_matrix",))
        if i % 5 == 1:
            ops += [("translate", u(-10, 10), u(-10, 10)), ("rotate", u(-0.4, 0.4))]
        elif i % 5 == 3:
            ops += [("scale", u(0.7, 1.3), u(0.7, 1.3))]
        cx, cy = u(0.2, 0.8) * size, u(0.2, 0.8) * size
        if k == 0:
            ops += [("move_to", cx, cy), ("arc", cx, cy, u(4, 40), u(0, 3), u(3, 9)), ("close_path",)]
        elif k == 1:
            ops += [("arc_negative", cx, cy, u(3, 30), u(0, 6), u(-3, 1))]
        elif k == 2:
            ops += [("move_to", cx, cy)]
            for j in range(3):
                ops.append(("elliptic_arc_to", u(0, size), u(0, size), j % 2 == 0, (i + j) % 2 == 0, u(8, 50),
                            u(8, 50), u(0, 3)))
        elif k == 3:
            ops += [("ellipse", u(5, 40), u(5, 40), cx, cy, u(0, 3))]
        elif k == 4:
            ops += [("rectangle", cx - 20, cy - 15, u(5, 50), u(5, 40)),
                    ("rounded_rectangle", u(0, size * 0.6), u(0, size * 0.6), u(10, 60), u(10, 60), u(1, 8))]
        elif k == 5:
            ops += [("move_to", cx, cy), ("quadratic_to", u(0, size), u(0, size), u(0, size), u(0, size)),
                    ("rel_quadratic_to", u(-30, 30), u(-30, 30), u(-30, 30), u(-30, 30)), ("close_path",)]
        elif k == 6:
            ops += [("move_to", cx, cy), ("rel_line_to", u(-40, 40), u(-40, 40)),
                    ("rel_curve_to", u(-40, 40), u(-40, 40), u(-40, 40), u(-40, 40), u(-40, 40), u(-40, 40)),
                    ("new_sub_path",), ("move_to", u(0, size), u(0, size)), ("line_to", u(0, size), u(0, size)),
                    ("rel_move_to", u(-20, 20), u(-20, 20)), ("rel_line_to", u(-30, 30), u(-30, 30)),
                    ("line_to", u(0, size), u(0, size))]
        else:
            ops += [("move_to", cx, cy)]
            for j in range(r.randint(3, 7)):
                ops.append(("line_to", u(0, size), u(0, size)))
            if i % 2:
                ops.append(("close_path",))
        ops += [("set_fill_rule", i % 2), ("set_opacity", 1.0 if i % 3 else u(0.3, 1.0)),
                ("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), u(0.3, 1.0))]
        ops.append(("set_operator", 3 if i % 11 == 10 else (0 if i % 13 == 12 else 2)))
        ops.append(("fill_preserve",) if i % 4 != 2 else ("stroke_preserve",))
        ops += [("set_operator", 2), ("set_line_width", u(0.5, 9)), ("set_line_join", (i // 2) % 3),
                ("set_line_cap", (i // 3) % 3), ("set_miter_limit", u(1.5, 12))]
        if i % 3 == 0:
            ops.append(("set_dash", [u(2, 12), u(1, 8), u(1, 9)][: 2 + (i % 2)], u(0, 10)))
        else:
            ops.append(("set_dash", [], 0.0))
        ops += [("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), u(0.4, 1.0))]
        ops.append(("stroke",) if i % 4 != 2 else ("fill",))
    return {"name": "api_mix", "width": size, "height": size, "samples": samples, "ops": ops, "paths": n_items}


def gradient_mix(n_items=14, size=144, seed=9, samples=4, radial=False):
    """Filled and stroked curves whose source is a linear gradient (with
    radial=True, every other one a radial gradient, some with the focus
    circle pulled inside the outer one by vkvg_pattern_edit_radial), under
    translated and rotated matrices and pattern matrices."""
    r = SplitMix64(seed)
    u = lambda lo, hi: lo + (hi - lo) * r.rnd()

    def stops():
        n = 2 + r.randint(0, 3)
        offs = sorted(r.rnd() for _ in range(n))
        offs[0], offs[-1] = 0.0, 1.0
        return [(o, r.rnd(), r.rnd(), r.rnd(), u(0.3, 1.0)) for o in offs]

    ops = [("set_source_rgb", 1.0, 1.0, 1.0), ("paint",),
           ("set_source_linear", 0.0, 0.0, float(size), 0.0, [(0.0, 0.1, 0.2, 0.9, 0.5), (1.0, 0.9, 0.5, 0.1, 0.5)],
            None), ("paint",)]
    for i in range(n_items):
        ops.append(("identity_matrix",))
        if i % 4 == 1:
            ops += [("translate", u(-8, 8), u(-8, 8)), ("rotate", u(-0.5, 0.5))]
        axis = i % 5
        x0, y0 = u(0, size), u(0, size)
        if axis == 0:
            x1, y1 = x0 + u(20, 100), y0
        elif axis == 1:
            x1, y1 = x0, y0 + u(20, 100)
        elif axis == 2:
            x1, y1 = x0 - u(20, 100), y0
        else:
            x1, y1 = u(0, size), u(0, size)
        pmat = (u(0.8, 1.2), u(-0.2, 0.2), u(-0.2, 0.2), u(0.8, 1.2), u(-5, 5), u(-5, 5)) if i % 3 == 2 else None
        ops.append(("move_to", u(0, size), u(0, size)))
        for _ in range(2):
            ops.append(("curve_to",) + tuple(u(0, size) for _ in range(6)))
        ops.append(("close_path",))
        if radial and i % 2:
            r1 = u(20, 90)
            r0 = u(0, r1 - 1) if i % 4 == 1 else u(0, 0.5 * r1)
            src = ("set_source_radial", x0, y0, r0, x0 + u(-0.4, 0.4) * r1, y0 + u(-0.4, 0.4) * r1, r1, stops(), pmat)
        else:
            src = ("set_source_linear", x0, y0, x1, y1, stops(), pmat)
        ops += [src, ("set_fill_rule", i % 2),
                ("set_opacity", 1.0 if i % 2 else u(0.4, 1.0)), ("fill_preserve",),
                ("set_line_width", u(1, 7)), ("set_line_join", i % 3)]
        if i % 3 == 0:
            ops += [("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), u(0.5, 1.0))]
        ops.append(("stroke",))
    return {"name": "radial_mix" if radial else "gradient_mix", "width": size, "height": size, "samples": samples,
            "ops": ops, "paths": n_items}


def clip_mix(n_items=10, size=128, seed=13, samples=4, flush_every=0):
    """Clip regions and the state stack: even-odd and non-zero clip paths,
    clip_preserve then fill, nested save / clip / restore, eight nested
    saves (the last two past the six stencil save bits), reset_clip, a clear
    with an active clip, restore re-snapping a gradient under a restored
    matrix, and the line join that vkvg_restore resets.  flush_every > 0
    flushes after that many items, so clip state crosses frames."""
    r = SplitMix64(seed)
    u = lambda lo, hi: lo + (hi - lo) * r.rnd()

    def blob(n=2):
        ops = [("move_to", u(0, size), u(0, size))]
        for _ in range(n):
            ops.append(("curve_to",) + tuple(u(-0.1 * size, 1.1 * size) for _ in range(6)))
        return ops + [("close_path",)]

    def rect(lo, hi):
        x, y = u(lo, hi), u(lo, hi)
        return [("rectangle", x, y, u(0.2, 0.6) * size, u(0.2, 0.6) * size)]

    def paint_layer():
        return [("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), u(0.5, 1.0)), ("paint",)]

    def shape_layer(i):
        return blob(2 + i % 2) + [("set_fill_rule", i % 2), ("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), u(0.4, 1.0)),
                                  ("fill_preserve",), ("set_line_width", u(1, 6)),
                                  ("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), u(0.6, 1.0)), ("stroke",)]

    ops = [("set_source_rgb", 1.0, 1.0, 1.0), ("paint",)]
    for i in range(n_items):
        mode = i % 5
        if mode == 0:  # one clip level: even-odd blob, paint and shapes inside
            ops += [("save",)] + blob(3) + [("set_fill_rule", 0), ("clip",)] + paint_layer() + shape_layer(i)
            ops += [("restore",)]
        elif mode == 1:  # nested: non-zero rect, then a blob with clip_preserve + fill
            ops += [("save",)] + rect(0, size * 0.5) + [("set_fill_rule", 1), ("clip",), ("save",)]
            ops += blob(2) + [("set_fill_rule", i % 2), ("clip_preserve",),
                              ("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), 0.8), ("fill",)]
            ops += paint_layer()[:1] + [("set_line_width", u(2, 8))] + blob(2) + [("stroke",), ("restore",)]
            ops += shape_layer(i) + [("restore",)] + shape_layer(i + 1)
        elif mode == 2:  # eight nested saves, each clipping further
            ops += [("set_line_join", 1)]
            for k in range(8):
                ops += [("save",)] + rect(-0.1 * size, 0.7 * size) + [("set_fill_rule", k % 2), ("clip",)]
                ops += [("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), 0.35), ("paint",)]
            for k in range(8):
                ops += [("restore",)] + shape_layer(i + k)[-6:]
            ops += [("set_line_width", 5.0)] + blob(2) + [("stroke",)]  # miter join after restore
        elif mode == 3:  # reset_clip inside a saved clip, gradient re-snapped by restore
            ops += [("identity_matrix",), ("translate", u(-10, 10), u(-10, 10))]
            ops += [("set_source_linear", 0.0, 0.0, float(size), u(0, size),
                     [(0.0, r.rnd(), r.rnd(), r.rnd(), 0.9), (1.0, r.rnd(), r.rnd(), r.rnd(), 0.6)], None)]
            ops += [("save",)] + blob(2) + [("clip",), ("paint",), ("rotate", u(-0.6, 0.6))]
            ops += [("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), 0.7), ("reset_clip",)] + blob(2) + [("fill",)]
            ops += [("restore",), ("paint",) if i % 2 else ("fill",), ("identity_matrix",)]
        else:  # clip without save, then a clear with the clip active, then reset
            ops += blob(2) + [("set_fill_rule", 0), ("clip",)] + paint_layer() + shape_layer(i)
            if i == 4:
                ops += [("clear",)] + paint_layer()
            ops += [("reset_clip",)] + shape_layer(i + 3)
        if flush_every and (i + 1) % flush_every == 0:
            ops.append(("flush",))
    return {"name": "clip_mix", "width": size, "height": size, "samples": samples, "ops": ops, "paths": n_items}


def vkvg_clip_cases(width=1024, height=800, samples=4):
    """The call sequences of vkvg's clip and save/restore demo programs
    (tests/clip.c: clipped_paint, clipped_paint2, clipped_transformed,
    clip_transformed, test_clip, test_clip2 for both fill rules where vkvg
    has both; tests/save_restore.c: twenty nested save / translate / stroke
    levels), one scene each on a fresh surface."""
    red, green, blue = ("set_source_rgb", 1.0, 0.0, 0.0), ("set_source_rgb", 0.0, 1.0, 0.0), \
        ("set_source_rgb", 0.0, 0.0, 1.0)
    base = lambda fr: [("set_fill_rule", fr), red, ("paint",)]
    rect = lambda x, y, w, h: ("rectangle", float(x), float(y), float(w), float(h))
    out = []
    for fr, tag in ((1, "nz"), (0, "eo")):
        out.append(("clipped_paint_" + tag, base(fr) + [green, rect(100, 100, 300, 200), ("clip",), ("paint",)]))
        out.append(("clipped_paint2_" + tag, base(fr) + [green, rect(100, 100, 300, 200), ("clip",), ("paint",),
                                                         ("reset_clip",), rect(200, 200, 300, 200), blue, ("paint",)]))
        out.append(("clipped_transformed_" + tag, base(fr) + [("rotate", 0.2), green, rect(100, 100, 300, 200),
                                                              ("clip",), ("paint",)]))
    out.append(("clip_transformed_nz", base(1) + [("rotate", 0.1), green, rect(100, 100, 300, 200), ("clip",),
                                                  ("paint",), ("translate", 200.0, 100.0), blue, ("paint",)]))
    star = [("move_to", 10.0, 10.0)] + [("line_to", float(x), float(y)) for x, y in
                                        ((400, 150), (900, 10), (700, 450), (900, 750), (500, 650), (100, 800),
                                         (150, 400))]
    out.append(("test_clip", [("clear",), ("set_fill_rule", 0)] + star +
                [("clip_preserve",), ("set_operator", 0), ("fill_preserve",), ("clip",), ("set_operator", 2), red,
                 ("paint",)]))
    out.append(("test_clip2", [("clear",), ("set_fill_rule", 1), rect(50, 50, 500, 500), ("clip",), red, ("paint",),
                               ("save",), rect(100, 100, 350, 350), ("clip",), ("save",),
                               ("set_source_rgb", 1.0, 1.0, 0.0), ("paint",), rect(200, 200, 200, 200), ("clip",),
                               green, ("paint",), ("restore",), rect(350, 350, 420, 420), blue, ("fill",),
                               ("restore",)]))
    rec = []
    for depth in range(1, 21):
        rec += [("save",), ("translate", 5.0, 5.0), rect(depth, depth, 200, 200), green, ("stroke",)]
    out.append(("save_restore", rec + [("restore",)] * 20))
    return [{"name": n, "width": width, "height": height, "samples": samples, "ops": ops, "paths": 0}
            for n, ops in out]


def vkvg_demo_cases(width=512, height=512, samples=4):
    """The call sequences of vkvg's single-sequence demo programs at their
    harness's default 512x512 surface (tests/common/test.c:38-39; the
    harness context of _initCtx, test.c:686-696: width 2, miter joins, butt
    caps, no dash, non-zero fill, cleared): tests/line_caps.c (the three
    caps on wide strokes, one stroke through several relative moves),
    tests/stroke.c (closed and open polylines, a wide line, a half-turn arc,
    a translucent wide diagonal, a rectangle), tests/fill.c (one concave
    polygon in the harness context), tests/fill_non_zero.c (a square with a
    square hole wound the other way, left empty under non-zero),
    tests/dashes.c (its first run: offset 0.2, four- and two-entry patterns
    with round caps and joins, a zero-length dash), tests/line_join.c (its
    three functions: wide round joins on closed polylines, zigzags with
    round then bevel joins under translations), tests/circles.c and
    tests/arcs.c (full and partial arcs of growing radii, arc_negative,
    scaled arcs, fill and stroke), tests/curve.c (its four fixed
    sequences: curves, a rounded rectangle of arcs, self-crossing wide
    strokes), tests/colinear.c, fill_and_stroke.c, simple_paint.c (paints
    under rotations and scales, with and without a path), compositing.c
    (translucent fills, opacity), radial_gradient.c, gradient.c (linear
    gradients on fills, strokes and paints, transformed, translucent stops),
    rect_fill.c, transform.c, bezier.c, gradient2.c and inverse_colinear.c,
    one scene each on a fresh surface."""
    import numpy as np

    rgba = lambda r, g, b, a: ("set_source_rgba", float(r), float(g), float(b), float(a))
    harness = [("set_line_width", 2.0), ("set_line_join", 0), ("set_line_cap", 0), ("set_dash", [], 0.0),
               ("set_fill_rule", 1), ("clear",)]
    out = []
    x, y, dx, dy = 20.0, 20.0, 40.0, 60.0
    caps = [rgba(0.9, 0.9, 0.9, 1), ("paint",), ("set_line_width", 30.0), rgba(0, 0, 0, 1),
            ("move_to", x, y), ("rel_line_to", 0.0, dy), ("stroke",), ("set_line_cap", 2),
            ("move_to", x + dx, y), ("rel_line_to", 0.0, dy), ("stroke",), ("set_line_cap", 1),
            ("move_to", x + 2 * dx, y), ("rel_line_to", 0.0, dy), ("rel_move_to", dx, -dy), ("rel_line_to", dx, dy),
            ("rel_move_to", dx, -dy / 2.0), ("rel_line_to", dx, 0.0), ("rel_move_to", dx, dy / 2.0),
            ("rel_line_to", dx, -dy), ("rel_move_to", dx, dy), ("rel_line_to", 0.0, -dy),
            ("rel_move_to", dx * 2.0, dy), ("rel_line_to", -dx, -dy), ("rel_move_to", dx * 3.0, dy / 2.0),
            ("rel_line_to", -dx, 0.0), ("stroke",), ("set_line_cap", 0), ("set_line_width", 1.0), rgba(1, 0, 0, 1),
            ("move_to", x, y), ("rel_line_to", 0.0, dy), ("rel_move_to", dx, -dy), ("rel_line_to", 0.0, dy),
            ("rel_move_to", dx, -dy), ("rel_line_to", 0.0, dy), ("stroke",)]
    out.append(("line_caps", caps))
    pif = 3.14159265358979323846
    stroke = [("set_line_width", 1.0), rgba(1, 0, 0, 1), ("move_to", 200.5, 200.5), ("line_to", 400.5, 200.5),
              ("line_to", 400.5, 400.5), ("line_to", 200.5, 400.5), ("close_path",), ("stroke",),
              rgba(0, 1, 0, 1), ("move_to", 300.5, 300.5), ("line_to", 500.5, 300.5), ("line_to", 500.5, 500.5),
              ("line_to", 300.5, 500.5), ("stroke",), rgba(0.5, 1, 0, 1), ("move_to", 320.5, 320.5),
              ("line_to", 520.5, 320.5), ("line_to", 520.5, 520.5), ("line_to", 320.5, 520.5), ("stroke",),
              ("set_line_width", 40.0), rgba(0.5, 0.6, 1, 1), ("move_to", 700.0, 475.0), ("line_to", 400.0, 475.0),
              ("stroke",), rgba(0, 0.5, 0.5, 0.5), ("move_to", 300.0, 200.0), ("arc", 200.0, 200.0, 100.0, 0.0, pif),
              ("stroke",), ("set_line_width", 20.0), rgba(0.1, 0.1, 0.1, 0.5), ("move_to", 100.0, 60.0),
              ("line_to", 400.0, 600.0), ("stroke",), rgba(1, 1, 1, 1), ("set_line_width", 1.0),
              ("rectangle", 600.5, 200.5, 100.0, 60.0), ("stroke",)]
    out.append(("stroke", stroke))
    fill = harness + [rgba(0.1, 0.9, 0.1, 1), ("move_to", 100.0, 100.0), ("rel_line_to", 50.0, 200.0),
                      ("rel_line_to", 150.0, -100.0), ("rel_line_to", 100.0, 200.0), ("rel_line_to", -100.0, 100.0),
                      ("rel_line_to", -10.0, -100.0), ("rel_line_to", -190.0, -50.0), ("close_path",), ("fill",)]
    out.append(("fill", fill))
    nz = [("save",), ("set_line_width", 30.0), ("set_fill_rule", 1), rgba(0.1, 0.9, 0.1, 1),
          ("move_to", 100.0, 100.0), ("rel_line_to", 200.0, 0.0), ("rel_line_to", 0.0, 150.0),
          ("rel_line_to", -200.0, 0.0), ("close_path",), ("move_to", 150.0, 150.0), ("rel_line_to", 0.0, 50.0),
          ("rel_line_to", 100.0, 0.0), ("rel_line_to", 0.0, -50.0), ("close_path",), ("fill",)]
    out.append(("fill_non_zero", nz))
    off = 0.2
    path_a = [("move_to", 50.0, 50.0), ("rel_line_to", 500.0, 0.0), ("rel_line_to", 0.0, 200.0),
              ("rel_line_to", 200.0, 0.0), ("rel_line_to", 0.0, 500.0), ("rel_line_to", -700.0, 0.0), ("close_path",)]
    path_b = [("move_to", 100.0, 100.0), ("rel_line_to", 400.0, 0.0), ("rel_line_to", 0.0, 200.0),
              ("rel_line_to", 200.0, 0.0), ("rel_line_to", 0.0, 400.0), ("rel_line_to", -600.0, 0.0), ("close_path",)]
    dashes = ([("clear",), ("set_source_rgb", 1.0, 1.0, 1.0), ("paint",), ("set_line_cap", 1), ("set_line_join", 1),
               ("set_dash", [100.0, 20.0, 20.0, 20.0], off), ("set_line_width", 4.0), ("set_source_rgb", 0.0, 0.0, 1.0)]
              + path_a + [("stroke",), ("set_dash", [0.0, 20.0], off), ("set_source_rgb", 0.0, 1.0, 0.0)] + path_b
              + [("stroke",), ("set_line_width", 10.0), ("set_source_rgb", 1.0, 0.0, 0.0),
                 ("set_dash", [80.0, 20.0], off), ("rectangle", 200.0, 300.0, 200.0, 200.0), ("stroke",)])
    out.append(("dashes", dashes))
    # tests/line_join.c: test, test2, test3
    x, y = 250.0, 150.0
    lj = [("set_line_width", 100.0), rgba(0, 1, 0, 1), ("set_line_join", 1), ("move_to", x, y),
          ("rel_line_to", -50.0, 30.0), ("rel_line_to", 0.0, 60.0), ("rel_line_to", 50.0, 30.0), ("close_path",),
          ("stroke",), rgba(0, 0, 1, 1), ("move_to", x + 250, y)]
    lj += [("rel_line_to", float(a), float(b)) for a, b in ((50, -30), (50, 0), (50, 30), (0, 60), (-50, 70),
                                                             (-50, 0), (-50, -70))]
    out.append(("line_join", lj + [("close_path",), ("stroke",)]))
    for name, starts, steps, shift in (
            ("line_join2", ((100, 100), (200, 600), (400, 100), (500, 600)),
             (((70, 50), (-70, 50)), ((70, -50), (-70, -50)), ((-70, 50), (70, 50)), ((-70, -50), (70, -50))), 5),
            ("line_join3", ((100, 100), (500, 200), (100, 400), (500, 500)),
             (((50, 70), (50, -70)), ((-50, 70), (-50, -70)), ((50, -70), (50, 70)), ((-50, -70), (-50, 70))), 4)):
        ops = [("set_fill_rule", 0), ("set_line_width", 30.0), ("set_line_join", 1), ("translate", -50.0, -50.0),
               ("set_source_rgb", 0.5, 0.0, 0.0)]
        for _ in range(2):
            for (sx, sy), (a, b) in zip(starts, steps):
                ops.append(("move_to", float(sx), float(sy)))
                for _ in range(shift):
                    ops += [("rel_line_to", float(a[0]), float(a[1])), ("rel_line_to", float(b[0]), float(b[1]))]
                ops.append(("stroke",))
            ops += [("set_line_join", 2), ("translate", 500.0 if name == "line_join2" else 450.0, 0.0)]
        out.append((name, ops))

    # tests/circles.c and tests/arcs.c (float32 pi as M_PIF; the circles' x
    # steps are exact in float32)
    def growing(yc, count, sweep):
        ops, xc = [], 2.0
        for i in range(1, count):
            xc += 0.5 * i
            ops.append(("arc", xc + 2, float(yc), 0.5 * i, 0.0, sweep))
            xc += 0.5 * i + 5
        return ops
    pif = float(np.float32(np.pi))
    white, black = ("set_source_rgb", 1.0, 1.0, 1.0), ("set_source_rgb", 0.0, 0.0, 0.0)
    out.append(("circles_fill_and_stroke", [("clear",), rgba(0, 0.1, 0.8, 0.5), ("set_line_width", 10.0),
                                            ("arc", 300.0, 300.0, 150.0, 0.0, pif * 2), ("fill_preserve",),
                                            ("stroke",)]))
    out.append(("circles_sizes", [("clear",), white] + growing(100, 40, pif * 2) + [("fill",)] +
                growing(200, 40, pif * 2) + [("stroke",), rgba(0, 0, 1, 0.4)] + growing(300, 40, pif * 2) +
                [("fill_preserve",), ("set_line_width", 5.0), ("stroke",)]))
    out.append(("circles_scaled_up", [("clear",), white, ("scale", 100.0, 100.0), ("arc", 2.0, 2.0, 0.5, 0.0, pif * 2),
                                      ("stroke",)]))
    out.append(("arcs_sizes", [white, ("paint",), black] + growing(100, 40, float(np.float32(pif * 1.5))) +
                [("stroke",)]))
    out.append(("arcs_scaled_up", [white, ("paint",), black, ("scale", 10.0, 10.0),
                                   ("arc", 20.0, 20.0, 2.0, 0.0, pif / 2), ("stroke",)]))
    arcs = [white, ("paint",), black, ("set_source_rgb", 1.0, 0.0, 1.0), ("set_line_width", 5.0),
            ("arc", 100.0, 100.0, 20.0, 0.0, pif / 2), ("stroke",), ("set_source_rgb", 0.0, 1.0, 1.0),
            ("arc_negative", 100.0, 100.0, 20.0, 0.0, pif / 2), ("stroke",), ("set_source_rgb", 1.0, 0.0, 1.0),
            ("arc", 100.0, 200.0, 20.0, pif / 2, 0.0), ("stroke",), ("set_source_rgb", 0.0, 1.0, 1.0),
            ("arc_negative", 100.0, 200.0, 20.0, pif / 2, 0.0), ("stroke",), ("set_source_rgb", 0.0, 0.0, 1.0),
            ("set_line_width", 10.0), ("arc", 350.0, 100.0, 40.0, 0.0, pif * 2), ("stroke",),
            ("set_source_rgb", 0.0, 1.0, 0.0), ("set_line_width", 1.0), ("arc", 150.0, 100.0, 3.5, 0.0, pif * 2),
            ("stroke",), ("arc", 200.0, 200.0, 10.0, 0.0, pif * 2), ("fill",), ("set_source_rgb", 1.0, 0.0, 0.0),
            ("scale", 3.0, 3.0), ("arc", 150.0, 100.0, 3.5, 0.0, pif * 2), ("stroke",),
            ("arc", 200.0, 200.0, 10.0, 0.0, pif * 2), ("fill",)]
    out.append(("arcs", arcs))
    # tests/curve.c: test3, test, curved_rect, test2 (the random ones need the
    # harness's generator and are left out)
    out.append(("curve_test3", [("clear",), ("set_line_width", 20.0), ("set_source_rgb", 1.0, 0.0, 0.0),
                                ("move_to", 80.0, 170.0), ("curve_to", 100.0, 170.0, 160.0, 171.0, 180.0, 170.0),
                                ("close_path",), ("stroke",)]))
    out.append(("curve_test", [("set_line_width", 20.0), ("scale", 2.0, 2.0), ("set_line_join", 2),
                               ("set_source_rgb", 0.5, 0.0, 0.0), ("translate", 200.0, 30.0),
                               ("arc", 200.0, 200.0, 20.0, 0.0, pif * 2), rgba(0.5, 0.0, 1.0, 0.5),
                               ("move_to", 100.0, 100.0), ("line_to", 200.0, 100.0),
                               ("curve_to", 250.0, 100.0, 300.0, 150.0, 300.0, 200.0), ("line_to", 300.0, 300.0),
                               ("curve_to", 300.0, 350.0, 250.0, 400.0, 200.0, 400.0), ("line_to", 100.0, 400.0),
                               ("curve_to", 50.0, 400.0, 10.0, 350.0, 10.0, 300.0), ("line_to", 10.0, 200.0),
                               ("curve_to", 10.0, 150.0, 50.0, 100.0, 100.0, 100.0), ("fill_preserve",),
                               rgba(0.1, 0.3, 0.7, 0.5), ("stroke",)]))
    x, y, w, h, r = 50.0, 50.0, 150.0, 140.0, 30.0
    hp, nhp = float(np.float32(np.pi / 2)), float(np.float32(-np.pi / 2))
    out.append(("curve_curved_rect", [("scale", 2.0, 2.0), ("set_line_width", 15.0), rgba(0, 0.5, 0.4, 1),
                                      ("move_to", x, y + r), ("arc", x + r, y + r, r, pif, nhp),
                                      ("line_to", x + w - r, y), ("arc", x + w - r, y + r, r, nhp, 0.0),
                                      ("line_to", x + w, y + h - r), ("arc", x + w - r, y + h - r, r, 0.0, hp),
                                      ("line_to", x + r, y + h), ("arc", x + r, y + h - r, r, hp, pif),
                                      ("line_to", x, y + r), ("close_path",), ("fill_preserve",),
                                      rgba(0.5, 0, 0, 0.5), ("stroke",)]))
    out.append(("curve_test2", [("move_to", 100.0, 400.0), ("curve_to", 100.0, 100.0, 600.0, 700.0, 600.0, 400.0),
                                ("curve_to", 1000.0, 100.0, 100.0, 800.0, 1000.0, 800.0),
                                ("curve_to", 1000.0, 500.0, 700.0, 500.0, 700.0, 100.0), ("close_path",),
                                rgba(1, 0, 0, 1), ("set_line_width", 40.0), ("stroke",)]))
    # tests/colinear.c, fill_and_stroke.c, simple_paint.c, compositing.c,
    # radial_gradient.c, gradient.c (vkvg's fragment stage ignores a
    # gradient's extend mode, so its vkvg_pattern_set_extend calls change
    # nothing and are left out)
    out.append(("colinear", [rgba(0.7, 0.7, 0.7, 1), ("paint",), rgba(0, 1, 0, 1), ("set_line_width", 10.0),
                             ("move_to", 100.0, 100.0), ("line_to", 100.0, 200.0), ("line_to", 100.0, 300.0),
                             ("stroke",)]))
    tri = lambda x0: [("move_to", x0, 100.0), ("rel_line_to", 50.0, -80.0), ("rel_line_to", 50.0, 80.0),
                      ("close_path",)]
    out.append(("fill_and_stroke", tri(100.0) + tri(300.0) + [("set_line_width", 10.0),
                                                              ("set_source_rgb", 0.0, 0.0, 1.0), ("fill_preserve",),
                                                              ("set_source_rgb", 1.0, 0.0, 0.0), ("stroke",)]))
    red = rgba(1, 0, 0, 1)
    rect = ("rectangle", 100.0, 100.0, 300.0, 200.0)
    for name, ops in (("paint", [rgba(1, 0, 0, 0.5), ("paint",)]),
                      ("paint_with_rotation", [("rotate", 45.0), red, ("paint",)]),
                      ("paint_with_scale", [("scale", 0.2, 0.2), red, ("paint",)]),
                      ("paint_rect", [red, rect, ("paint",)]),
                      ("paint_rect_with_rotation", [("rotate", 45.0), red, rect, ("paint",)]),
                      ("paint_rect_with_scale", [("scale", 0.2, 0.2), red, rect, ("paint",)])):
        out.append(("simple_" + name, harness + ops))
    out.append(("compositing", [("clear",), rgba(1, 0, 0, 0.5), ("rectangle", 100.0, 100.0, 200.0, 200.0), ("fill",),
                                rgba(0, 0, 1, 0.5), ("rectangle", 200.0, 200.0, 200.0, 200.0), ("fill",)]))
    out.append(("opacity", [("clear",), red, ("rectangle", 100.0, 100.0, 200.0, 200.0), ("fill",),
                            ("set_opacity", 0.5), rgba(0, 0, 1, 1), ("rectangle", 200.0, 200.0, 200.0, 200.0),
                            ("fill",)]))
    out.append(("radial_gradient", [("set_source_radial", 250.0, 250.0, 0.0, 300.0, 300.0, 260.0,
                                     [(0.0, 1.0, 0.0, 0.0, 1.0), (0.5, 0.0, 1.0, 0.0, 1.0),
                                      (1.0, 0.0, 0.0, 0.0, 1.0)]), ("paint",)]))
    rgb3 = [(0.0, 1.0, 0.0, 0.0, 1.0), (0.5, 0.0, 1.0, 0.0, 1.0), (1.0, 0.0, 0.0, 1.0, 1.0)]
    grad = lambda x0: ("set_source_linear", x0, 0.0, 300.0, 0.0, rgb3)
    gp = [("rectangle", 0.0, 0.0, 400.0, 460.0), grad(0.0), ("fill",), ("rectangle", 100.0, 200.0, 50.0, 50.0),
          grad(100.0), ("fill",), ("rectangle", 10.0, 10.0, 300.0, 50.0),
          ("set_source_linear", 10.0, 0.0, 300.0, 0.0, [(0.0, 0.0, 0.0, 1.0, 0.0), (1.0, 1.0, 0.0, 0.0, 1.0)]),
          ("fill",), ("rectangle", 400.0, 200.0, 50.0, 50.0), grad(400.0), ("fill",),
          ("rectangle", 500.0, 200.0, 50.0, 50.0), grad(500.0), ("fill",)]
    out.append(("gradient_paint", harness + gp))
    out.append(("gradient_paint_repeat", harness + [grad(0.0), ("paint",)]))
    out.append(("gradient_test", harness + [grad(0.0), ("rectangle", 100.0, 100.0, 200.0, 200.0),
                                            ("set_line_width", 20.0), ("stroke",)]))
    out.append(("gradient_test2", harness + [("set_source_rgb", 1.0, 0.0, 0.0), ("paint",), ("set_line_width", 20.0),
                                             ("set_source_linear", 100.0, 0.0, 300.0, 0.0,
                                              [(0.0, 1.0, 1.0, 1.0, 1.0), (1.0, 1.0, 1.0, 0.0, 0.0)]),
                                             ("rectangle", 100.0, 100.0, 200.0, 200.0), ("fill",)]))
    out.append(("gradient_transform", harness + [("translate", 200.0, 100.0), ("rotate", 0.5), ("set_line_width", 20.0),
                                                 ("set_source_linear", 0.0, 0.0, 400.0, 0.0, rgb3),
                                                 ("rectangle", 0.0, 0.0, 400.0, 200.0), ("stroke",)]))
    out.append(("gradient_alpha", harness + [("set_source_rgb", 0.0, 1.0, 0.0), ("paint",),
                                             ("set_source_linear", 10.0, 0.0, 300.0, 0.0,
                                              [(1.0, 1.0, 0.0, 0.0, 0.5), (1.0, 1.0, 0.0, 0.0, 0.5)]),
                                             ("rectangle", 10.0, 10.0, 300.0, 200.0), ("fill",)]))
    # tests/rect_fill.c (both fill rules) and tests/transform.c
    # (cairo_tests' first run: rotation 0.002, the 512x512 surface's centre)
    sq = [rgba(0, 0, 1, 0.5), ("rectangle", 100.0, 100.0, 200.0, 200.0), ("fill",),
          ("rectangle", 200.0, 200.0, 200.0, 200.0), rgba(1, 0, 0, 0.5), ("fill",)]
    out.append(("rect_fill", [("clear",), ("set_fill_rule", 1)] + sq))
    out.append(("rect_fill_evenodd", [("clear",), ("set_fill_rule", 0)] + sq))
    a0, a1 = -100.0, 100.0
    rounded = [("move_to", a0, 0.0), ("curve_to", a0, a0, a0, a0, 0.0, a0), ("curve_to", a1, a0, a1, a0, a1, 0.0),
               ("curve_to", a1, a1, a1, a1, 0.0, a1), ("curve_to", a0, a1, a0, a1, a0, 0.0), ("close_path",),
               ("set_source_rgb", 0.5, 0.5, 1.0), ("fill_preserve",), rgba(0.5, 0, 0, 0.5),
               ("set_line_width", 10.0), ("stroke",)]
    out.append(("transform_cairo", [("set_fill_rule", 0), rgba(1, 1, 1, 1), ("paint",), ("set_line_width", 10.0),
                                    ("set_source_rgb", 0.0, 0.0, 1.0), ("translate", width / 2.0, height / 2.0),
                                    ("rotate", float(np.float32(0.002))),
                                    ("arc", 0.0, 0.0, 150.0, 0.0, float(np.float32(np.pi * 1.5))), ("stroke",)]
                + rounded))
    # tests/bezier.c (its first frame: the self-crossing cubic, no point
    # hovered, at 4 samples instead of its 8)
    pts = ((150.0, 150.0), (500.0, 340.0), (470.0, 150.0), (160.0, 350.0))
    bz = [("clear",), ("set_line_width", 10.0), ("set_line_join", 0), ("set_line_cap", 0), ("move_to",) + pts[0],
          ("curve_to",) + pts[1] + pts[2] + pts[3], rgba(1, 0, 0, 0.3), ("stroke",), ("flush",),
          ("set_line_width", 1.0), rgba(0.5, 0.5, 0.5, 0.6)]
    for px, py in pts:
        bz += [("arc", px, py, 5.0, 0.0, pif * 2), ("fill_preserve",), ("stroke",)]
    out.append(("bezier", bz + [("stroke",)]))
    # tests/gradient2.c (its first frame, linear; and its radial pattern type)
    stops4 = [(0.0, 1.0, 0.0, 0.0, 0.5), (0.3, 0.0, 1.0, 0.0, 0.5), (0.6, 0.0, 0.0, 1.0, 0.5), (1.0, 0.0, 0.0, 0.0, 0.5)]
    marks = [("set_dash", [], 0.0), ("set_line_width", 1.0)]
    for px, py in ((150.0, 150.0), (250.0, 150.0)):
        marks += [rgba(1.0, 0.5, 0.5, 0.9), ("arc", px, py, 7.0, 0.0, pif * 2), ("fill_preserve",), ("stroke",)]
    out.append(("gradient2_linear", [("clear",), ("set_source_linear", 150.0, 150.0, 250.0, 150.0, stops4),
                                     ("paint",)] + marks))
    out.append(("gradient2_radial", [("clear",), ("set_source_radial", 125.0, 125.0, 20.0, 150.0, 150.0, 100.0,
                                                  stops4), ("paint",)] + marks))
    # tests/inverse_colinear.c: its first frame (a wide mitered polyline
    # with sharp turns) and the settings its keys switch: closed with bevel
    # joins; round joins and caps with its {0, 60} dash; arcs (arc_negative)
    # at both ends
    ipts = ((150.0, 150.0), (200.0, 300.0), (250.0, 150.0), (280.0, 350.0))
    a15, api = float(np.float32(pif * 1.5)), pif

    def inv(join, cap, closed, dash, arcs):
        ops = [("clear",)] + ([("set_dash", [0.0, 60.0], 0.0)] if dash else []) + [
            rgba(1, 0, 0, 0.3), ("set_line_width", 50.0), ("set_line_join", join), ("set_line_cap", cap),
            ("set_miter_limit", 10.0)]
        ops.append(("arc_negative", ipts[0][0], ipts[0][1], 200.0, a15, api) if arcs else ("move_to",) + ipts[0])
        ops += [("line_to",) + p for p in ipts[1:-1]]
        ops.append(("arc_negative", ipts[-1][0], ipts[-1][1], 200.0, a15, api) if arcs else ("line_to",) + ipts[-1])
        return ops + ([("close_path",)] if closed else []) + [("stroke",)]
    out.append(("inverse_colinear", inv(0, 0, False, False, False)))
    out.append(("inverse_colinear_closed_bevel", inv(2, 0, True, False, False)))
    out.append(("inverse_colinear_round_dash", inv(1, 1, False, True, False)))
    out.append(("inverse_colinear_arcs", inv(0, 0, False, False, True)))
    return [{"name": n, "width": width, "height": height, "samples": samples, "ops": ops, "paths": 0}
            for n, ops in out]


def surface_mix(n_items=12, size=128, seed=23, samples=4):
    """Surface sources: two small drawn surfaces (one of odd size) used as
    sources with vkvg_set_source_surface offsets and as surface patterns with
    every extend mode, nearest and bilinear filtering and pattern matrices,
    under translated, rotated and scaled matrices, with opacity, inside
    save / restore, and after a gradient source (whose surface-size offset a
    later pattern source inherits)."""
    r = SplitMix64(seed)
    u = lambda lo, hi: lo + (hi - lo) * r.rnd()

    def source(w, h):
        ops = [("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), 0.6), ("paint",)]
        for _ in range(4):
            ops += [("move_to", u(0, w), u(0, h))]
            ops += [("curve_to",) + tuple(u(-0.2, 1.2) * (w if k % 2 == 0 else h) for k in range(6))]
            ops += [("close_path",), ("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), u(0.5, 1.0)), ("fill_preserve",),
                    ("set_line_width", u(1, 4)), ("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), 1.0), ("stroke",)]
        return {"width": w, "height": h, "ops": ops}

    def shape():
        ops = [("move_to", u(0, size), u(0, size))]
        for _ in range(2):
            ops.append(("curve_to",) + tuple(u(-0.1, 1.1) * size for _ in range(6)))
        return ops + [("close_path",)]

    ops = [("set_source_rgb", 0.9, 0.9, 0.85), ("paint",)]
    for i in range(n_items):
        ops.append(("identity_matrix",))
        if i % 3 == 1:
            ops += [("translate", u(-20, 20), u(-20, 20)), ("rotate", u(-0.7, 0.7))]
        elif i % 3 == 2:
            ops += [("scale", u(0.6, 1.8), u(0.6, 1.8))]
        src = i % 2
        if i % 4 == 0:
            ops.append(("set_source_surface", src, u(-10, size * 0.7), u(-10, size * 0.7)))
        else:
            pmat = (u(0.5, 1.5), u(-0.3, 0.3), u(-0.3, 0.3), u(0.5, 1.5), u(-9, 9), u(-9, 9)) if i % 3 else None
            ops.append(("set_source_surface_pattern", src, i % 4, 4 if i % 5 < 3 else 0, pmat))
        ops.append(("set_opacity", 1.0 if i % 3 else u(0.3, 0.9)))
        if i == 5:
            ops += [("save",), ("set_source_linear", 0.0, 0.0, float(size), 0.0,
                                [(0.0, 1.0, 0.0, 0.0, 1.0), (1.0, 0.0, 0.0, 1.0, 1.0)], None),
                    ("set_source_surface_pattern", 1, 1, 4, None)]
        ops += shape() + [("set_fill_rule", i % 2), ("fill_preserve",), ("set_line_width", u(2, 9)), ("stroke",)]
        if i == 5:
            ops += [("restore",), ("rectangle", 4.0, 4.0, 30.0, 20.0), ("fill",)]
        if i == n_items - 1:
            ops += [("set_opacity", 0.5), ("paint",)]
    return {"name": "surface_mix", "width": size, "height": size, "samples": samples, "ops": ops,
            "paths": n_items, "sources": [source(48, 40), source(33, 17)]}


def play(ctx, ops, sources=()):
    """Replay a scene's calls on a context object with vkvg method names;
    surface sources name their surface by its index in `sources`."""
    for op in ops:
        name, args = op[0], op[1:]
        if name in ("set_source_surface", "set_source_surface_pattern"):
            getattr(ctx, name)(sources[args[0]], *args[1:])
        elif name == "set_dash":
            ctx.set_dash(args[0], args[1])
        elif name == "set_source_linear":
            ctx.set_source_linear(*args)
        elif name == "set_source_radial":
            ctx.set_source_radial(*args)
        elif name == "set_matrix":
            ctx.set_matrix(args[0])
        else:
            getattr(ctx, name)(*args)


# vkvg recording command codes (src/recording/vkvg_record_internal.h:28-90),
# the wire format of vkvg_gb300_replay_stream
CMD = {
    "new_path": 0x0101, "new_sub_path": 0x0102, "close_path": 0x0103, "move_to": 0x0104, "line_to": 0x0105,
    "rectangle": 0x0106, "arc": 0x0107, "arc_negative": 0x0108, "curve_to": 0x010A, "quadratic_to": 0x010B,
    "elliptic_arc_to": 0x010C, "set_line_width": 0x1101, "set_miter_limit": 0x1102, "set_line_join": 0x1103,
    "set_line_cap": 0x1104, "set_operator": 0x1105, "set_fill_rule": 0x1106, "set_dash": 0x1107,
    "translate": 0x2001, "rotate": 0x2002, "scale": 0x2003, "identity_matrix": 0x2005, "set_matrix": 0x2006,
    "rel_move_to": 0x0504, "rel_line_to": 0x0505, "rel_curve_to": 0x050A, "rel_quadratic_to": 0x050B,
    "paint": 0x0201, "fill": 0x0202, "stroke": 0x0203, "clear": 0x0206, "fill_preserve": 0x0602,
    "stroke_preserve": 0x0603, "set_source_rgb": 0x0801, "set_source_rgba": 0x0802, "set_source_color": 0x0803,
    "save": 0x0001, "restore": 0x0002, "clip": 0x0204, "reset_clip": 0x0205, "clip_preserve": 0x0604,
}


def encode(ops):
    """scene calls -> (cmds uint32[], args float32[]) for vkvg_gb300_replay_stream"""
    import struct

    import numpy as np

    cmds, args = [], []
    for op in ops:
        name, a = op[0], op[1:]
        cmds.append(CMD[name])
        if name == "set_dash":
            args += [float(len(a[0])), float(a[1])] + [float(v) for v in a[0]]
        elif name == "set_matrix":
            args += [float(v) for v in a[0]]
        elif name == "set_source_color":
            args.append(struct.unpack("<f", struct.pack("<I", a[0]))[0])
        else:
            args += [float(v) for v in a]
    return np.array(cmds, np.uint32), np.array(args, np.float32)


def svg_document(seed=31, n_shapes=40, size=240, quirks=False):
    """A seeded SVG document exercising what vkvg's SVG path reads: every
    path command (absolute and relative, implicit repeats, arcs with packed
    flags), rect / rounded rect / circle / ellipse / line / polyline /
    polygon, nested groups with transform lists (matrix, translate, scale,
    rotate about a point, skewX, skewY), style attributes and style="...",
    colours as #rgb, #rrggbb, rgb(), rgb(%) and names (known and unknown),
    opacities, stroke widths with units, linear and radial gradients with
    stops (one reached through xlink:href), display:none, and a viewBox with
    preserveAspectRatio.  With quirks, some empty-element tags get a space
    before their closing '/>', some values trailing spaces, and some path
    data a trailing newline.  (Whitespace before the '>' of a start tag is
    not generated: vkvg's parser takes the string terminator for whitespace
    there and reads on into the following tags.)  Returns the document text
    (bytes)."""
    r = SplitMix64(seed)
    u = lambda lo, hi: lo + (hi - lo) * r.rnd()
    pick = lambda seq: seq[r.randint(0, len(seq) - 1)]

    def num(v):
        k = r.randint(0, 5)
        if k == 0:
            return "%.0f" % v
        if k == 1:
            return ("%.3e" % v)
        if k == 2 and abs(v) < 1:
            return ("%.3f" % v).replace("0.", ".", 1)
        return "%.2f" % v

    def color():
        k = r.randint(0, 6)
        if k == 0:
            return "#%x%x%x" % (r.randint(0, 15), r.randint(0, 15), r.randint(0, 15))
        if k == 1:
            return "rgb(%d,%d,%d)" % (r.randint(0, 255), r.randint(0, 255), r.randint(0, 255))
        if k == 2:
            return "rgb(%d%%, %d%%, %d%%)" % (r.randint(0, 100), r.randint(0, 100), r.randint(0, 100))
        if k == 3:
            return pick(["red", "green", "blue", "yellow", "cyan", "magenta", "black", "grey", "white", "orange"])
        return "#%02x%02x%02x" % (r.randint(0, 255), r.randint(0, 255), r.randint(0, 255))

    def paint():
        k = r.randint(0, 9)
        if k == 0:
            return "none"
        if k == 1:
            return "url(#lg%d)" % r.randint(0, 2)
        if k == 2:
            return "url(#rg0)"
        return color()

    def transform():
        fs = []
        for _ in range(r.randint(1, 3)):
            k = r.randint(0, 5)
            if k == 0:
                fs.append("translate(%s,%s)" % (num(u(-30, 30)), num(u(-30, 30))))
            elif k == 1:
                fs.append("scale(%s)" % num(u(0.6, 1.4)) if r.randint(0, 1) else
                          "scale(%s %s)" % (num(u(0.6, 1.4)), num(u(0.6, 1.4))))
            elif k == 2:
                fs.append("rotate(%s)" % num(u(-40, 40)) if r.randint(0, 1) else
                          "rotate(%s %s %s)" % (num(u(-40, 40)), num(u(0, size)), num(u(0, size))))
            elif k == 3:
                fs.append("skewX(%s)" % num(u(-20, 20)))
            elif k == 4:
                fs.append("skewY(%s)" % num(u(-20, 20)))
            else:
                fs.append("matrix(%s)" % " ".join(num(v) for v in (u(0.7, 1.2), u(-0.3, 0.3), u(-0.3, 0.3),
                                                                     u(0.7, 1.2), u(-20, 20), u(-20, 20))))
        return " ".join(fs)

    def style_attrs():
        out = []
        if r.randint(0, 2) == 0:
            decl = ["fill:%s" % paint(), "stroke:%s" % paint(), "stroke-width:%s" % num(u(0.5, 6))]
            if r.randint(0, 1):
                decl.append("fill-opacity: %s" % num(u(0.2, 1)))
            out.append('style="%s"' % "; ".join(decl[:r.randint(1, len(decl))]))
        else:
            if r.randint(0, 3):
                out.append('fill="%s"' % paint())
            if r.randint(0, 1):
                out.append('stroke="%s"' % paint())
                out.append('stroke-width="%s%s"' % (num(u(0.5, 5)), pick(["", "px", "pt", "mm", "%"])))
            if r.randint(0, 3) == 0:
                out.append('stroke-opacity="%s"' % num(u(0.2, 1)))
        if r.randint(0, 4) == 0:
            out.append('opacity="%s"' % num(u(0.3, 1)))
        if r.randint(0, 4) == 0:
            out.append('transform="%s"' % transform())
        if r.randint(0, 25) == 0:
            out.append('display="none"')
        return " ".join(out)

    def path_data():
        d = ["M%s %s" % (num(u(0, size)), num(u(0, size)))]
        for _ in range(r.randint(2, 7)):
            c = pick("LlHhVvCcSsQqTtAa")
            k = {"L": 2, "H": 1, "V": 1, "C": 6, "S": 4, "Q": 4, "T": 2, "A": 7}[c.upper()]
            reps = r.randint(1, 2)
            args = []
            for _ in range(reps):
                if c.upper() == "A":
                    args += [num(u(5, 60)), num(u(5, 60)), num(u(-90, 90))]
                    flags = "%d%d" % (r.randint(0, 1), r.randint(0, 1))
                    args.append(flags if r.randint(0, 1) else " ".join(flags))
                    args += [num(u(-40, 40) if c == "a" else u(0, size)), num(u(-40, 40) if c == "a" else u(0, size))]
                else:
                    args += [num(u(-40, 40) if c.islower() else u(0, size)) for _ in range(k)]
            sep = pick([" ", ","])
            d.append(c + sep.join(args))
        if r.randint(0, 1):
            d.append(pick(["Z", "z"]))
        if r.randint(0, 3) == 0:
            d.append("m%s %s l%s %s %s %s z" % tuple(num(u(-30, 30)) for _ in range(6)))
        return "".join(x + pick([" ", "", "\n"]) for x in d)

    def shape():
        k = r.randint(0, 7)
        a = style_attrs()
        if k <= 1:
            return '<path id="p%d" d="%s" %s/>' % (r.randint(0, 999), path_data(), a)
        if k == 2:
            rr = ' rx="%s"' % num(u(0, 15)) if r.randint(0, 1) else ""
            rr += ' ry="%s"' % num(u(0, 15)) if r.randint(0, 2) == 0 else ""
            return '<rect x="%s" y="%s" width="%s" height="%s"%s %s/>' % (
                num(u(0, size)), num(u(0, size)), num(u(5, 90)), num(u(5, 90)), rr, a)
        if k == 3:
            return '<circle cx="%s" cy="%s" r="%s" %s/>' % (num(u(0, size)), num(u(0, size)), num(u(3, 50)), a)
        if k == 4:
            return '<ellipse cx="%s" cy="%s" rx="%s" ry="%s" %s/>' % (
                num(u(0, size)), num(u(0, size)), num(u(3, 60)), num(u(3, 40)), a)
        if k == 5:
            return '<line x1="%s" y1="%s" x2="%s" y2="%s" %s/>' % tuple(
                [num(u(0, size)) for _ in range(4)] + [a])
        pts = " ".join("%s,%s" % (num(u(0, size)), num(u(0, size))) for _ in range(r.randint(3, 7)))
        return '<%s points="%s" %s/>' % ("polyline" if k == 6 else "polygon", pts, a)

    vb = r.randint(0, 3)
    root = ['width="%d" height="%d"' % (size, size)]
    if vb:
        root.append('viewBox="%s %s %s %s"' % (num(u(-20, 20)), num(u(-20, 20)), num(u(size * 0.8, size * 1.3)),
                                               num(u(size * 0.8, size * 1.3))))
        root.append('preserveAspectRatio="%s"' % pick(["xMidYMid meet", "xMinYMax slice", "none", "xMaxYMin"]))
    out = ['<?xml version="1.0" encoding="UTF-8"?>', "<!-- seeded test document -->",
           '<svg xmlns="http://www.w3.org/2000/svg" xmlns:xlink="http://www.w3.org/1999/xlink" %s>' % " ".join(root),
           "<defs>"]
    for g in range(3):
        if g == 2:
            out.append('<linearGradient id="lg2" xlink:href="#lg0" x1="0" y1="0" x2="1" y2="1"/>')
            continue
        out.append('<linearGradient id="lg%d" x1="%s" y1="0" x2="1" y2="%s">' % (g, num(u(0, 0.5)), num(u(0, 1))))
        for _ in range(r.randint(2, 4)):
            off = u(0, 1)
            if r.randint(0, 1):
                out.append('<stop offset="%s" stop-color="%s" stop-opacity="%s"/>' % (num(off), color(), num(u(0.3, 1))))
            else:
                out.append('<stop offset="%d%%" style="stop-color:%s"/>' % (int(off * 100), color()))
        out.append("</linearGradient>")
    out.append('<radialGradient id="rg0" cx="50%" cy="50%" r="50%">')
    out.append('<stop offset="0" stop-color="%s"/><stop offset="1" stop-color="%s"/>' % (color(), color()))
    out.append("</radialGradient></defs>")
    depth = 0
    for i in range(n_shapes):
        if r.randint(0, 5) == 0 and depth < 3:
            out.append(('<g id="g%d" %s' % (i, style_attrs())).rstrip() + ">")
            depth += 1
        out.append(shape())
        if depth and r.randint(0, 4) == 0:
            out.append("</g>")
            depth -= 1
    out += ["</g>"] * depth + ["</svg>"]
    text = "\n".join(out)
    if quirks:
        q = []
        for part in text.split("\n"):
            k = r.randint(0, 5)
            if k == 0 and part.endswith('"/>'):
                part = part[:-3] + '" />'
            elif k == 1 and part.startswith('" '):
                part = "\n" + part
            elif k == 2 and ' d="' in part:
                part = part.replace('" ', '  " ', 1)
            q.append(part)
        text = "\n".join(q)
    return text.encode()


def batch_scenes(seed=2, n_surfaces=64, max_paths=20000, min_paths=100, max_segs=2000, max_side=2048,
                 samples=4):
    """The uneven batch: n_surfaces independent surfaces, side log-uniform in
    [256, max_side] rounded to a multiple of 16; paths per surface
    Pareto(alpha 1.2) clipped to [min_paths, max_paths]; segments per path
    log-uniform in [3, max_segs], 70% cubics, 20% lines, 10% arcs of radius
    U[2, 200] px; path bounding boxes log-uniform from 4 px to the surface;
    60% filled, 30% filled then stroked, 10% stroked, width U[0.5, 12].
    Returns a list of scenes (one per surface)."""
    import math

    r = SplitMix64(seed)
    u = lambda lo, hi: lo + (hi - lo) * r.rnd()
    logu = lambda lo, hi: math.exp(u(math.log(lo), math.log(hi)))
    out = []
    for k in range(n_surfaces):
        side = max(16, int(round(logu(256, max_side) / 16.0)) * 16)
        n_paths = int(min(max_paths, max(min_paths, min_paths * (1.0 - r.rnd()) ** (-1.0 / 1.2))))
        ops = [("set_source_rgb", 1.0, 1.0, 1.0), ("paint",)]
        for i in range(n_paths):
            bw = logu(4, side)
            bx, by = u(0, side - bw), u(0, side - bw)
            pt = lambda: (bx + u(0, bw), by + u(0, bw))
            nseg = int(logu(3, max_segs))
            ops.append(("move_to",) + pt())
            for _ in range(nseg):
                t = r.rnd()
                if t < 0.7:
                    ops.append(("curve_to",) + pt() + pt() + pt())
                elif t < 0.9:
                    ops.append(("line_to",) + pt())
                else:
                    rad = min(u(2, 200), bw)
                    cx, cy = pt()
                    a0 = u(0, 2 * math.pi)
                    ops.append(("arc", cx, cy, rad, a0, a0 + u(0.3, 2 * math.pi)))
            ops.append(("close_path",))
            kind = r.rnd()
            ops.append(("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), u(0.3, 1.0)))
            if kind < 0.6:
                ops.append(("fill",))
            else:
                if kind < 0.9:
                    ops.append(("fill_preserve",))
                    ops.append(("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), u(0.5, 1.0)))
                ops += [("set_line_width", u(0.5, 12)), ("stroke",)]
        out.append({"name": "batch%d" % k, "width": side, "height": side, "samples": samples, "ops": ops,
                    "paths": n_paths})
    return out


def np_rnd(seed, start, n):
    """outputs start+1 .. start+n of SplitMix64(seed) as floats in [0, 1)
    (SplitMix64's i-th output is mix(seed + i * gamma), so a block is one
    vector operation)"""
    import numpy as np

    with np.errstate(over="ignore"):
        z = np.uint64(seed & MASK64) + (np.arange(start + 1, start + n + 1, dtype=np.uint64) *
                                        np.uint64(0x9E3779B97F4A7C15))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(40)).astype(np.float64) * (1.0 / 16777216.0)


def batch_streams(seed=2, n_surfaces=64, max_paths=20000, min_paths=100, max_segs=2000, max_side=2048,
                  paths_scale=1.0):
    """The uneven batch (64 independent surfaces in one job), generated as
    vkvg command streams for vkvg_gb300_replay_stream: side log-uniform in
    [256, max_side] rounded to a multiple of 16; paths per surface
    Pareto(alpha 1.2) clipped to [min_paths, max_paths] (times paths_scale);
    segments per path log-uniform in [3, max_segs], 70% cubics, 20% lines and
    10% arcs of radius U[2, 200] px (at most the box); path bounding boxes
    log-uniform from 4 px to the surface; 60% of paths filled, 30% filled
    then stroked, 10% stroked, width U[0.5, 12], colours uniform with alpha
    U[0.3, 1].  Each surface is cleared to opaque white.  Returns one dict
    per surface: width, height, cmds (uint32), args (float32), paths."""
    import math

    import numpy as np

    top = SplitMix64(seed)
    C_ = CMD
    out = []
    for k in range(n_surfaces):
        s = top.next()
        a = np_rnd(s, 0, 2)
        side = max(16, int(round(math.exp(math.log(256) + (math.log(max_side) - math.log(256)) * a[0]) / 16.0)) * 16)
        n_paths = int(min(max_paths, max(min_paths, min_paths * (1.0 - a[1]) ** (-1.0 / 1.2))))
        n_paths = max(1, int(n_paths * paths_scale))
        P = np_rnd(s, 2, n_paths * 12).reshape(n_paths, 12)
        bw = np.exp(math.log(4) + (math.log(side) - math.log(4)) * P[:, 0])
        bx, by = P[:, 1] * (side - bw), P[:, 2] * (side - bw)
        nseg = np.exp(math.log(3) + (math.log(max_segs) - math.log(3)) * P[:, 3]).astype(np.int64)
        kind = P[:, 4]
        total = int(nseg.sum())
        S = np_rnd(s, 2 + n_paths * 12, total * 8).reshape(total, 8)
        pb = np.repeat(np.arange(n_paths), nseg)
        sbw, sbx, sby = bw[pb], bx[pb], by[pb]
        t = S[:, 0]
        cub, lin = t < 0.7, (t >= 0.7) & (t < 0.9)
        arc = ~(cub | lin)
        seg_args = np.zeros((total, 6))
        seg_args[:, 0::2] = sbx[:, None] + S[:, 1:7:2] * sbw[:, None]
        seg_args[:, 1::2] = sby[:, None] + S[:, 2:7:2] * sbw[:, None]
        rad = np.minimum(2.0 + 198.0 * S[:, 3], sbw)
        a0 = 2 * math.pi * S[:, 4]
        arc_args = np.stack([seg_args[:, 0], seg_args[:, 1], rad, a0, a0 + 0.3 + (2 * math.pi - 0.3) * S[:, 5],
                             np.zeros(total)], 1)
        seg_args = np.where(arc[:, None], arc_args, seg_args)
        nargs = np.where(cub, 6, np.where(lin, 2, 5))
        mask = np.arange(6)[None, :] < nargs[:, None]
        seg_cmd = np.where(cub, C_["curve_to"], np.where(lin, C_["line_to"], C_["arc"])).astype(np.uint32)
        seg_flat = seg_args[mask]
        seg_off = np.concatenate([[0], np.cumsum(nargs)])
        seg0 = np.concatenate([[0], np.cumsum(nseg)])
        cmds, args = [np.array([C_["set_source_rgb"], C_["paint"]], np.uint32)], [np.array([1.0, 1.0, 1.0])]
        for i in range(n_paths):
            c = [C_["move_to"]]
            x0, y0 = bx[i] + P[i, 5] * bw[i], by[i] + P[i, 6] * bw[i]
            cmds.append(np.array([C_["move_to"]], np.uint32))
            args.append(np.array([x0, y0]))
            cmds.append(seg_cmd[seg0[i]:seg0[i + 1]])
            args.append(seg_flat[seg_off[seg0[i]]:seg_off[seg0[i + 1]]])
            rgba = P[i, 7:11].copy()
            rgba[3] = 0.3 + 0.7 * rgba[3]
            c = [C_["close_path"], C_["set_source_rgba"]]
            g = list(rgba)
            width = 0.5 + 11.5 * P[i, 11]
            if kind[i] < 0.6:
                c.append(C_["fill"])
            elif kind[i] < 0.9:
                c += [C_["fill_preserve"], C_["set_source_rgba"], C_["set_line_width"], C_["stroke"]]
                g += [rgba[2], rgba[0], rgba[1], 0.5 + 0.5 * P[i, 9], width]
            else:
                c += [C_["set_line_width"], C_["stroke"]]
                g += [width]
            cmds.append(np.array(c, np.uint32))
            args.append(np.array(g))
        out.append({"name": "batch%d" % k, "width": side, "height": side, "paths": n_paths,
                    "cmds": np.concatenate(cmds).astype(np.uint32), "args": np.concatenate(args).astype(np.float32)})
    return out


def decode(cmds, args):
    """command stream -> scene calls (the inverse of encode for the codes
    batch_streams and glyph_streams emit)"""
    names = {v: k for k, v in CMD.items()}
    nargs = {"move_to": 2, "line_to": 2, "curve_to": 6, "quadratic_to": 4, "arc": 5, "close_path": 0,
             "set_source_rgb": 3, "set_source_rgba": 4, "paint": 0, "fill": 0, "fill_preserve": 0, "stroke": 0,
             "set_line_width": 1, "set_line_join": 1, "set_fill_rule": 1}
    ops, a = [], 0
    ints = ("set_line_join", "set_fill_rule")
    for c in cmds:
        name = names[int(c)]
        n = nargs[name]
        ops.append((name,) + tuple(int(v) if name in ints else float(v) for v in args[a:a + n]))
        a += n
    return ops


# ------------------------------------------------------------------ analytic

AN_LINE, AN_CUBIC = 1, 3
AN_FILL, AN_STROKE = 1, 2


def analytic_scene(seed=3, n_paths=128, n_cubics=8, size=256, w_min=0.5, w_max=4.0):
    """Scene of the differentiable analytic-coverage mode: a size x size fp32
    RGBA canvas on an opaque white background; n_paths closed paths of
    n_cubics cubic Beziers each, control points uniform in [0,size)^2; per
    path a colour with straight RGBA U[0,1) premultiplied by its alpha, a
    NON_ZERO fill and a stroke of width U[w_min, w_max) in the same colour.
    The differentiable benchmark uses seed 3 for the optimised paths and
    seed 4 for the target image.  Returns the scene description and its
    parameters (float32 arrays)."""
    import numpy as np

    r = SplitMix64(seed)
    ncp = n_paths * n_cubics * 3
    ctrl = np.array([r.rnd() * size for _ in range(2 * ncp)], np.float32).reshape(ncp, 2)
    colors = np.zeros((n_paths, 4), np.float32)
    widths = np.zeros(n_paths, np.float32)
    for p in range(n_paths):
        rgb = [r.rnd() for _ in range(3)]
        a = r.rnd()
        colors[p] = [rgb[0] * a, rgb[1] * a, rgb[2] * a, a]
        widths[p] = w_min + r.rnd() * (w_max - w_min)
    scene = {
        "width": size, "height": size, "background": np.ones(4, np.float32),
        "path_ncontours": np.ones(n_paths, np.uint32),
        "path_flags": np.full(n_paths, AN_FILL | AN_STROKE, np.uint32),
        "contour_nseg": np.full(n_paths, n_cubics, np.uint32),
        "seg_kind": np.full(n_paths * n_cubics, AN_CUBIC, np.uint8),
    }
    return scene, {"ctrl": ctrl, "colors": colors, "widths": widths}


def analytic_glyph_scene(seed=5, n_outlines=200000, n_strokes=20000, size=4096, size_min=8.0, size_max=48.0):
    """The large glyph configuration in the analytic mode's terms: a size x
    size fp32 canvas on white; n_outlines glyph-like outlines of quadratic
    Beziers (outline size U[size_min, size_max) px, 1-3 contours of 6-40
    quads, the outer contour counter-clockwise on screen and the holes inside
    it clockwise), each a fill layer (NON_ZERO); then n_strokes closed chains
    of 3-8 quads as stroke layers of width U[1, 3) (the analytic mode strokes
    closed contours with bevel joints).  Each path's colour is the scene's
    linear gradient (two random RGBA stops along a random axis) at the path's
    first point, premultiplied.  Every quadratic is degree-elevated to the
    cubic with the same curve (control points p, p + 2/3 (q - p),
    p' + 2/3 (q - p'), exact), so the mode's cubic segments carry it; quad
    holds the outline control points (on-curve P, off-curve Q, next on-curve
    index) and elevate / elevate_adjoint map them to the cubic control
    points and gradients back.  Random values are splitmix64 outputs drawn in
    blocks (np_rnd).  Returns (scene, params, quad)."""
    import numpy as np

    pos = [0]

    def take(n):
        v = np_rnd(seed, pos[0], n)
        pos[0] += n
        return v

    g = take(12)
    gx0, gy0, gx1, gy1 = g[0] * size, g[1] * size, g[2] * size, g[3] * size
    c0 = np.array([g[4], g[5], g[6], 0.5 + 0.5 * g[7]])
    c1 = np.array([g[8], g[9], g[10], 0.5 + 0.5 * g[11]])
    o = take(4 * n_outlines).reshape(n_outlines, 4)
    cx, cy = o[:, 0] * size, o[:, 1] * size
    osz = size_min + (size_max - size_min) * o[:, 2]
    ncont = 1 + np.minimum((o[:, 3] * 3).astype(np.int64), 2)
    nc = int(ncont.sum())
    cont_out = np.repeat(np.arange(n_outlines), ncont)
    first = np.zeros(nc, bool)
    first[np.concatenate([[0], np.cumsum(ncont)[:-1]])] = True
    c = take(4 * nc).reshape(nc, 4)
    nq = 6 + np.minimum((c[:, 0] * 35).astype(np.int64), 34)
    half = osz[cont_out] / 2
    rad = np.where(first, half, half * (0.2 + 0.2 * c[:, 1]))
    off = np.where(first, 0.0, half * 0.35)
    ang = c[:, 2] * 2 * np.pi
    ccx, ccy = cx[cont_out] + off * np.cos(ang), cy[cont_out] + off * np.sin(ang)
    sgn = np.where(first, -1.0, 1.0)
    nqt = int(nq.sum())
    qc = np.repeat(np.arange(nc), nq)
    k = np.arange(nqt) - np.repeat(np.cumsum(nq) - nq, nq)
    q = take(3 * nqt).reshape(nqt, 3)
    th = (k + 0.3 * (q[:, 0] - 0.5)) * (2 * np.pi / nq[qc])
    th_c = (k + 0.5) * (2 * np.pi / nq[qc])
    r_on, r_off = rad[qc] * (0.7 + 0.3 * q[:, 1]), rad[qc] * (0.7 + 0.45 * q[:, 2])
    P = np.stack([ccx[qc] + r_on * np.cos(sgn[qc] * th), ccy[qc] + r_on * np.sin(sgn[qc] * th)], 1)
    Q = np.stack([ccx[qc] + r_off * np.cos(sgn[qc] * th_c), ccy[qc] + r_off * np.sin(sgn[qc] * th_c)], 1)
    nxt = np.arange(nqt) + 1
    last = np.cumsum(nq) - 1
    nxt[last] = last - nq + 1
    path_ncont = list(ncont)
    cont_nseg = list(nq)
    flags = [AN_FILL] * n_outlines
    widths = np.ones(n_outlines + n_strokes, np.float32)
    path_start = np.concatenate([[0], np.cumsum(np.add.reduceat(nq, np.concatenate([[0], np.cumsum(ncont)[:-1]])))[:-1]])
    starts = [P[path_start]]
    if n_strokes:
        st = take(5 * n_strokes).reshape(n_strokes, 5)
        ns = 3 + np.minimum((st[:, 0] * 6).astype(np.int64), 5)
        nst = int(ns.sum())
        sk = np.arange(nst) - np.repeat(np.cumsum(ns) - ns, ns)
        si = np.repeat(np.arange(n_strokes), ns)
        w = take(4 * nst).reshape(nst, 4)
        step = 6.0 + 12.0 * st[:, 3]
        hd = st[:, 4] * 2 * np.pi
        sx0, sy0 = st[:, 1] * size, st[:, 2] * size
        hh = hd[si] + np.cumsum(0.8 * (w[:, 0] - 0.5))
        ex = sx0[si] + np.cumsum(step[si] * np.cos(hh))
        ey = sy0[si] + np.cumsum(step[si] * np.sin(hh))
        b0 = np.cumsum(ns) - ns
        ex = ex - np.repeat(ex[b0] - sx0 - step * np.cos(hh[b0]), ns)
        ey = ey - np.repeat(ey[b0] - sy0 - step * np.sin(hh[b0]), ns)
        # on-curve points: the chain's start then its joints; the last quad
        # closes the contour back to the start
        SP = np.stack([np.where(sk == 0, np.repeat(sx0, ns), np.roll(ex, 1)),
                       np.where(sk == 0, np.repeat(sy0, ns), np.roll(ey, 1))], 1)
        SN = np.stack([np.where(sk == ns[si] - 1, np.repeat(sx0, ns), ex), np.where(sk == ns[si] - 1, np.repeat(sy0, ns), ey)], 1)
        SQ = 0.5 * (SP + SN) + np.stack([0.4 * step[si] * (w[:, 1] - 0.5), 0.4 * step[si] * (w[:, 2] - 0.5)], 1)
        snxt = nqt + np.arange(nst) + 1
        slast = nqt + np.cumsum(ns) - 1
        snxt[slast - nqt] = slast - ns + 1
        P = np.concatenate([P, SP])
        Q = np.concatenate([Q, SQ])
        nxt = np.concatenate([nxt, snxt])
        path_ncont += [1] * n_strokes
        cont_nseg += list(ns)
        flags += [AN_STROKE] * n_strokes
        widths[n_outlines:] = 1.0 + 2.0 * w[b0, 3]
        starts.append(SP[b0])
    starts = np.concatenate(starts)
    # colour: the gradient at the path's first point (smoothstep between the stops)
    dx, dy = gx1 - gx0, gy1 - gy0
    t = np.clip(((starts[:, 0] - gx0) * dx + (starts[:, 1] - gy0) * dy) / max(dx * dx + dy * dy, 1e-9), 0.0, 1.0)
    t = t * t * (3 - 2 * t)
    col = c0[None, :] * (1 - t[:, None]) + c1[None, :] * t[:, None]
    colors = np.concatenate([col[:, :3] * col[:, 3:], col[:, 3:]], 1).astype(np.float32)
    nseg = len(P)
    scene = {
        "width": size, "height": size, "background": np.ones(4, np.float32),
        "path_ncontours": np.array(path_ncont, np.uint32), "path_flags": np.array(flags, np.uint32),
        "contour_nseg": np.array(cont_nseg, np.uint32), "seg_kind": np.full(nseg, AN_CUBIC, np.uint8),
    }
    quad = {"P": P.astype(np.float32), "Q": Q.astype(np.float32), "nxt": nxt.astype(np.int64)}
    return scene, {"ctrl": elevate(quad), "colors": colors, "widths": widths}, quad


def elevate(quad, P=None, Q=None):
    """cubic control points [segments * 3][2] of the quadratic segments
    (start p, p + 2/3 (q - p), p' + 2/3 (q - p') with p' the next on-curve
    point), in float32, or in float64 when P or Q is float64"""
    import numpy as np

    P = quad["P"] if P is None else P
    Q = quad["Q"] if Q is None else Q
    dt = np.float64 if np.float64 in (np.asarray(P).dtype, np.asarray(Q).dtype) else np.float32
    P, Q = np.asarray(P, dt), np.asarray(Q, dt)
    t = dt(2.0 / 3.0)
    out = np.empty((len(P), 3, 2), dt)
    out[:, 0] = P
    np.subtract(Q, P, out=out[:, 1])
    out[:, 1] *= t
    out[:, 1] += P
    Pn = P[quad["nxt"]]
    np.subtract(Q, Pn, out=out[:, 2])
    out[:, 2] *= t
    out[:, 2] += Pn
    return out.reshape(-1, 2)


def elevate_adjoint(quad, g):
    """gradients of the on-curve and off-curve points from the gradients of
    the cubic control points (the transpose of elevate)"""
    import numpy as np

    g = np.asarray(g, np.float64).reshape(-1, 3, 2)
    n = len(g)
    gP = g[:, 0] + g[:, 1] / 3.0
    nxt = quad["nxt"]
    gP[:, 0] += np.bincount(nxt, g[:, 2, 0], n) / 3.0
    gP[:, 1] += np.bincount(nxt, g[:, 2, 1], n) / 3.0
    gQ = (2.0 / 3.0) * (g[:, 1] + g[:, 2])
    return gP, gQ


def glyph_streams(seed=5, n_outlines=200000, n_strokes=20000, size=4096, size_min=8.0, size_max=48.0):
    """The large glyph scene as a command stream: a size x size surface, MSAA
    4, which the caller paints white and then sets the gradient source on
    before replaying the stream; n_outlines glyph-like closed outlines of quadratic
    Beziers - outline size U[size_min, size_max) px, 1-3 contours, 6-40 quads
    per contour; the first contour runs counter-clockwise on screen and the
    others (holes, inside it) clockwise - filled NON_ZERO; then n_strokes
    open strokes of 3-8 quads, width U[1,3), round joins.  Every draw uses
    one linear gradient between two random RGBA stops along a random axis,
    which the caller sets as the source before replaying ("gradient": x0,
    y0, x1, y1 and two (offset, r, g, b, a) stops).  Random values are
    splitmix64 outputs (np_rnd), drawn in blocks so that the scene builds in
    seconds.  Returns cmds, args, the gradient and the counts."""
    import numpy as np

    C = CMD
    pos = [0]

    def take(n):
        v = np_rnd(seed, pos[0], n)
        pos[0] += n
        return v

    g = take(12)
    grad = (g[0] * size, g[1] * size, g[2] * size, g[3] * size,
            [(0.0, g[4], g[5], g[6], 0.5 + 0.5 * g[7]), (1.0, g[8], g[9], g[10], 0.5 + 0.5 * g[11])])
    # per outline: centre, size, contour count; per contour: quad count
    o = take(4 * n_outlines).reshape(n_outlines, 4)
    cx, cy = o[:, 0] * size, o[:, 1] * size
    osz = size_min + (size_max - size_min) * o[:, 2]
    ncont = 1 + np.minimum((o[:, 3] * 3).astype(np.int64), 2)
    nc = int(ncont.sum())
    cont_out = np.repeat(np.arange(n_outlines), ncont)
    first = np.zeros(nc, bool)
    first[np.concatenate([[0], np.cumsum(ncont)[:-1]])] = True
    c = take(4 * nc).reshape(nc, 4)
    nq = 6 + np.minimum((c[:, 0] * 35).astype(np.int64), 34)
    # contour frame: outer contours span the outline, holes a fifth to two
    # fifths of it, placed inside it
    half = osz[cont_out] / 2
    rad = np.where(first, half, half * (0.2 + 0.2 * c[:, 1]))
    off = np.where(first, 0.0, half * 0.35)
    ang = c[:, 2] * 2 * np.pi
    ccx = cx[cont_out] + off * np.cos(ang)
    ccy = cy[cont_out] + off * np.sin(ang)
    sgn = np.where(first, -1.0, 1.0)  # y down: decreasing screen angle is counter-clockwise
    nqt = int(nq.sum())
    qc = np.repeat(np.arange(nc), nq)
    k = np.arange(nqt) - np.repeat(np.cumsum(nq) - nq, nq)
    q = take(3 * nqt).reshape(nqt, 3)
    th = (k + 0.3 * (q[:, 0] - 0.5)) * (2 * np.pi / nq[qc])
    th_c = (k + 0.5) * (2 * np.pi / nq[qc])
    r_on = rad[qc] * (0.7 + 0.3 * q[:, 1])
    r_off = rad[qc] * (0.7 + 0.45 * q[:, 2])
    px = ccx[qc] + r_on * np.cos(sgn[qc] * th)
    py = ccy[qc] + r_on * np.sin(sgn[qc] * th)
    ox = ccx[qc] + r_off * np.cos(sgn[qc] * th_c)
    oy = ccy[qc] + r_off * np.sin(sgn[qc] * th_c)
    # stream: per contour move_to(p0), quads to p1 .. p_{n-1}, p0, close_path;
    # per outline one fill after its contours
    nxt = np.arange(nqt) + 1
    last = np.cumsum(nq) - 1
    nxt[last] = last - nq + 1
    cmd_list, arg_list = [], []
    head = [(C["set_fill_rule"], [0.0])]
    for cm, a in head:
        cmd_list.append(np.array([cm], np.uint32))
        arg_list.append(np.array(a, np.float32))
    # cmds per contour: move_to, nq quads, close_path; fill after the last contour of an outline
    ncmd = nq + 2 + np.where(np.r_[first[1:], True], 1, 0)
    cbase = np.concatenate([[0], np.cumsum(ncmd)[:-1]])
    cm = np.empty(int(ncmd.sum()), np.uint32)
    cm[cbase] = C["move_to"]
    qi = np.repeat(cbase + 1, nq) + k
    cm[qi] = C["quadratic_to"]
    cm[cbase + 1 + nq] = C["close_path"]
    has_fill = np.r_[first[1:], True]
    cm[(cbase + 2 + nq)[has_fill]] = C["fill"]
    nargs = np.zeros(len(cm), np.int64)
    nargs[cbase] = 2
    nargs[qi] = 4
    abase = np.concatenate([[0], np.cumsum(nargs)[:-1]])
    ar = np.empty(int(nargs.sum()), np.float32)
    s0 = np.repeat(np.cumsum(nq) - nq, 1)
    ar[abase[cbase]] = px[s0]
    ar[abase[cbase] + 1] = py[s0]
    ar[abase[qi]] = ox
    ar[abase[qi] + 1] = oy
    ar[abase[qi] + 2] = px[nxt]
    ar[abase[qi] + 3] = py[nxt]
    cmd_list.append(cm)
    arg_list.append(ar)
    # strokes: open chains of 3-8 quads, width U[1,3), round joins
    if n_strokes:
        st = take(5 * n_strokes).reshape(n_strokes, 5)
        ns = 3 + np.minimum((st[:, 0] * 6).astype(np.int64), 5)
        nst = int(ns.sum())
        sk = np.arange(nst) - np.repeat(np.cumsum(ns) - ns, ns)
        si = np.repeat(np.arange(n_strokes), ns)
        w = take(4 * nst).reshape(nst, 4)
        step = 6.0 + 12.0 * st[:, 3]
        hd = st[:, 4] * 2 * np.pi
        sx0, sy0 = st[:, 1] * size, st[:, 2] * size
        hh = hd[si] + np.cumsum(0.8 * (w[:, 0] - 0.5))
        ex = sx0[si] + np.cumsum(step[si] * np.cos(hh))
        ey = sy0[si] + np.cumsum(step[si] * np.sin(hh))
        # restart the running sums at every stroke
        b0 = np.cumsum(ns) - ns
        ex = ex - np.repeat(ex[b0] - sx0 - step * np.cos(hh[b0]), ns)
        ey = ey - np.repeat(ey[b0] - sy0 - step * np.sin(hh[b0]), ns)
        prx = np.where(sk == 0, np.repeat(sx0, ns), np.roll(ex, 1))
        pry = np.where(sk == 0, np.repeat(sy0, ns), np.roll(ey, 1))
        qx = 0.5 * (prx + ex) + 0.4 * step[si] * (w[:, 1] - 0.5)
        qy = 0.5 * (pry + ey) + 0.4 * step[si] * (w[:, 2] - 0.5)
        width = 1.0 + 2.0 * w[b0, 3]
        per = ns + 4  # set_line_width, set_line_join, move_to, quads, stroke
        sb = np.concatenate([[0], np.cumsum(per)[:-1]])
        scm = np.empty(int(per.sum()), np.uint32)
        scm[sb] = C["set_line_width"]
        scm[sb + 1] = C["set_line_join"]
        scm[sb + 2] = C["move_to"]
        sq = np.repeat(sb + 3, ns) + sk
        scm[sq] = C["quadratic_to"]
        scm[sb + 3 + ns] = C["stroke"]
        sna = np.zeros(len(scm), np.int64)
        sna[sb] = 1
        sna[sb + 1] = 1
        sna[sb + 2] = 2
        sna[sq] = 4
        sab = np.concatenate([[0], np.cumsum(sna)[:-1]])
        sar = np.empty(int(sna.sum()), np.float32)
        sar[sab[sb]] = width
        sar[sab[sb + 1]] = 1.0  # VKVG_LINE_JOIN_ROUND
        sar[sab[sb + 2]] = sx0
        sar[sab[sb + 2] + 1] = sy0
        sar[sab[sq]] = qx
        sar[sab[sq] + 1] = qy
        sar[sab[sq] + 2] = ex
        sar[sab[sq] + 3] = ey
        cmd_list.append(scm)
        arg_list.append(sar)
    return {"width": size, "height": size, "samples": 4, "cmds": np.concatenate(cmd_list),
            "args": np.concatenate(arg_list), "gradient": grad, "outlines": n_outlines, "strokes": n_strokes,
            "contours": nc, "quads": nqt + (int(ns.sum()) if n_strokes else 0)}


def glyph_scene(**kw):
    """glyph_streams as a scene of calls: white paint, the gradient source,
    then the stream's calls"""
    s = glyph_streams(**kw)
    x0, y0, x1, y1, stops = s["gradient"]
    ops = [("set_source_rgb", 1.0, 1.0, 1.0), ("paint",),
           ("set_source_linear", float(x0), float(y0), float(x1), float(y1),
            [tuple(float(v) for v in st) for st in stops])]
    ops += decode(s["cmds"], s["args"])
    return {"name": "glyphs", "width": s["width"], "height": s["height"], "samples": 4, "ops": ops,
            "paths": s["outlines"] + s["strokes"]}
