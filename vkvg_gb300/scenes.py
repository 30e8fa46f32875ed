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


def gradient_mix(n_items=14, size=144, seed=9, samples=4):
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
        ops += [("set_source_linear", x0, y0, x1, y1, stops(), pmat), ("set_fill_rule", i % 2),
                ("set_opacity", 1.0 if i % 2 else u(0.4, 1.0)), ("fill_preserve",),
                ("set_line_width", u(1, 7)), ("set_line_join", i % 3)]
        if i % 3 == 0:
            ops += [("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), u(0.5, 1.0))]
        ops.append(("stroke",))
    return {"name": "gradient_mix", "width": size, "height": size, "samples": samples, "ops": ops, "paths": n_items}


def play(ctx, ops):
    """Replay a scene's calls on a context object with vkvg method names."""
    for op in ops:
        name, args = op[0], op[1:]
        if name == "set_dash":
            ctx.set_dash(args[0], args[1])
        elif name == "set_source_linear":
            ctx.set_source_linear(*args)
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
