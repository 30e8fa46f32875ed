"""vkvg_svg_render (src/nsvg/vkvg_nsvg.c:82-136) restated over parsed shape
records (vkvg_gb300.Svg.shapes(), nsvg_ref.parse() or a fixture), driving any
context with vkvg method names (test infrastructure: the oracle side of the
SVG parity tests)."""
import numpy as np

F = np.float32
PAINT_NONE, PAINT_COLOR, PAINT_LINEAR = 0, 1, 2


def _set_color(ctx, c, alpha):
    """_svg_set_color: the ABGR word's channels over 255 in fp32, alpha times
    the shape opacity"""
    a = F(c >> 24 & 255) / F(255)
    b = F(c >> 16 & 255) / F(255)
    g = F(c >> 8 & 255) / F(255)
    r = F(c & 255) / F(255)
    ctx.set_source_rgba(float(r), float(g), float(b), float(a * F(alpha)))


def render(ctx, shapes, sub_id=None):
    ctx.save()
    ctx.set_fill_rule(0)  # VKVG_FILL_RULE_EVEN_ODD
    ctx.set_source_rgba(0.0, 0.0, 0.0, 1.0)
    for sh in shapes:
        if sub_id is not None and sh["id"] != sub_id:
            continue
        ctx.new_path()
        o = sh["opacity"]
        ctx.set_line_width(float(sh["stroke_width"]))
        for pts, closed in sh["paths"]:
            ctx.move_to(float(pts[0, 0]), float(pts[0, 1]))
            for i in range(1, len(pts), 3):
                q = pts[i:i + 3].reshape(-1)
                ctx.curve_to(*[float(v) for v in q])
            if closed:
                ctx.close_path()
        if sh["fill_type"] in (PAINT_COLOR, PAINT_LINEAR):
            _set_color(ctx, sh["fill_color"], o)
        if sh["fill_type"] != PAINT_NONE:
            if sh["stroke_type"] == PAINT_NONE:
                ctx.fill()
                continue
            ctx.fill_preserve()
        if sh["stroke_type"] in (PAINT_COLOR, PAINT_LINEAR):
            _set_color(ctx, sh["stroke_color"], o)
        ctx.stroke()
    ctx.restore()
