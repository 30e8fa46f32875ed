"""Differentiable analytic coverage (include/vkvg_gb300.h vkvg_gb300_analytic_*).

CPU: the FP64 reference (oracle/vko_analytic.c, tests/analytic_ref.py)
against exact areas computed independently here (polygon clipping per pixel),
its flattening against vkvg's own recorder restatement, and its hand-derived
adjoint against central finite differences of its own forward.

GPU (-m gpu): the CUDA path against the FP64 reference on the same scenes:
flattened points bit-exact (the subdivision is vkvg's, taken in fp32 on both
sides), canvas and loss within fp32 rounding, gradients within 1e-3 relative
error of the FP64 adjoint and of FP64 central finite differences (h = 1e-3)
on 256 random parameters of the 256x256, 128-path scene, the torch.autograd
wrapper (harness only), Adam steps, ragged and degenerate inputs, and the
point-buffer growth path."""
import numpy as np
import pytest

import analytic_ref as ar
from vkvg_gb300 import scenes

# canvas: fp32 compositing of up to 256 layers against the double reference
CANVAS_TOL = 2e-4
# gradients: the target of the differentiable mode
GRAD_TOL = 1e-3


def _one_path(ctrl_pts, kinds, flags=scenes.AN_FILL, size=16, contours=None):
    contours = contours or [len(kinds)]
    sc = {"width": size, "height": size, "background": np.ones(4, np.float32),
          "path_ncontours": np.array([len(contours)], np.uint32), "path_flags": np.array([flags], np.uint32),
          "contour_nseg": np.array(contours, np.uint32), "seg_kind": np.array(kinds, np.uint8)}
    return sc, np.asarray(ctrl_pts, np.float64)


def _clip_area(poly, x0, y0):
    """exact area of a convex-or-not polygon clipped to the unit pixel
    [x0,x0+1]x[y0,y0+1] (Sutherland-Hodgman, then the shoelace formula): the
    signed area integral of the winding number over the pixel"""
    def clip(pts, inside, inter):
        out = []
        for i in range(len(pts)):
            a, b = pts[i - 1], pts[i]
            ia, ib = inside(a), inside(b)
            if ib:
                if not ia:
                    out.append(inter(a, b))
                out.append(b)
            elif ia:
                out.append(inter(a, b))
        return out

    def ix(c):
        return lambda a, b: (c, a[1] + (b[1] - a[1]) * (c - a[0]) / (b[0] - a[0]))

    def iy(c):
        return lambda a, b: (a[0] + (b[0] - a[0]) * (c - a[1]) / (b[1] - a[1]), c)

    pts = [tuple(p) for p in poly]
    for inside, inter in ((lambda p: p[0] >= x0, ix(x0)), (lambda p: p[0] <= x0 + 1, ix(x0 + 1)),
                          (lambda p: p[1] >= y0, iy(y0)), (lambda p: p[1] <= y0 + 1, iy(y0 + 1))):
        pts = clip(pts, inside, inter)
        if not pts:
            return 0.0
    s = 0.0
    for i in range(len(pts)):
        (xa, ya), (xb, yb) = pts[i - 1], pts[i]
        s += xa * yb - xb * ya
    return -0.5 * s  # the oracle's orientation: clockwise on screen is positive


@pytest.mark.parametrize("poly", [
    [(1.25, 2.5), (5.75, 2.5), (5.75, 6.0), (1.25, 6.0)],
    [(3.1, 0.4), (9.7, 4.2), (6.3, 11.9), (0.6, 7.7)],
    [(2.2, 2.9), (12.4, 5.3), (4.8, 13.1)],
    [(-3.5, 4.25), (7.5, -2.0), (18.0, 9.5), (6.2, 17.3)],  # crosses every canvas side
])
def test_fill_area_matches_exact_clipping(poly):
    """per-pixel signed area of a polygon = exact polygon-pixel intersection"""
    sc, ctrl = _one_path(poly, [scenes.AN_LINE] * len(poly))
    R = ar.Reference(sc)
    _, _, A = R.forward(ctrl, np.array([[0, 0, 0, 1.0]]), np.array([1.0]), area=True)
    want = np.array([[_clip_area(poly, i, j) for i in range(16)] for j in range(16)])
    assert np.abs(A[0] - want).max() < 1e-12


def test_stroke_area_is_rectangles_plus_bevels():
    """the stroke's raw area is the sum of its rectangles (length x width) and
    bevel triangles (h^2 sin(turn) / 2), whatever the pixel grid"""
    poly = np.array([(3.3, 4.1), (12.6, 3.2), (11.1, 12.7), (4.4, 10.2)])
    w = 1.7
    sc, ctrl = _one_path(poly, [scenes.AN_LINE] * 4, flags=scenes.AN_STROKE, size=24)
    R = ar.Reference(sc)
    _, _, A = R.forward(ctrl, np.array([[0, 0, 0, 1.0]]), np.array([w]), area=True)
    n = len(poly)
    want = 0.0
    for k in range(n):
        d = poly[(k + 1) % n] - poly[k]
        want += np.hypot(*d) * w
        da, db = poly[k] - poly[k - 1], poly[(k + 1) % n] - poly[k]
        s = abs(da[0] * db[1] - da[1] * db[0]) / (np.hypot(*da) * np.hypot(*db))
        want += 0.5 * (w / 2) ** 2 * s
    assert abs(A[0].sum() - want) < 1e-9


def test_flattening_is_vkvg_recorders(vko):
    """the reference's fp32 points are the points vkvg's path recorder keeps
    for move_to, curve_to x n, close_path (oracle restatement of
    src/vkvg_context.c:341-584)"""
    scene, par = scenes.analytic_scene(seed=7, n_paths=6, n_cubics=5, size=200)
    R = ar.Reference(scene)
    f32, f64, seg = R.flatten(par["ctrl"])
    assert np.abs(f32 - f64).max() < 1e-3
    s = vko.OracleSurface(200, 200, 1)
    ctx = s.context()
    ctx.keep_draws(1)
    cp = par["ctrl"].astype(np.float32)
    for p in range(6):
        base = p * 15
        ctx.move_to(*cp[base])
        for k in range(5):
            c = [cp[base + 3 * k + 1], cp[base + 3 * k + 2], cp[base + (3 * k + 3) % 15]]
            ctx.curve_to(*c[0], *c[1], *c[2])
        ctx.close_path()
        ctx.fill()
    draws = ctx.draws()
    got = np.concatenate([d["points"] for d in draws])
    assert got.shape == f32.shape and np.array_equal(got.view(np.uint32), f32.view(np.uint32))


def _small():
    scene, par = scenes.analytic_scene(seed=3, n_paths=8, n_cubics=4, size=64)
    _, tpar = scenes.analytic_scene(seed=4, n_paths=8, n_cubics=4, size=64)
    R = ar.Reference(scene)
    target, _ = R.forward(tpar["ctrl"], tpar["colors"], tpar["widths"])
    return R, par, target


def _sample(R, n, rng):
    g = np.concatenate([np.zeros(n // 2), np.ones(n // 4), 2 * np.ones(n - n // 2 - n // 4)]).astype(np.uint32)
    idx = np.concatenate([rng.choice(2 * R.nctrl, n // 2, replace=False),
                          rng.choice(4 * R.npaths, n // 4, replace=False),
                          rng.choice(R.npaths, n - n // 2 - n // 4, replace=len(g) - n // 2 - n // 4 > R.npaths)])
    return g, idx.astype(np.uint32)


def _pick(grads, g, idx):
    d_ctrl, d_col, d_w = grads
    return np.array([d_ctrl.reshape(-1)[i] if k == 0 else d_col.reshape(-1)[i] if k == 1 else d_w[i]
                     for k, i in zip(g, idx)])


def rel_err(a, b, floor):
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def smooth_fd(R, par, target, g, idx, h=1e-3):
    """FP64 central differences at h, and which of them measure a derivative:
    the flattening must not change within h, and the differences at h and
    h/10 must agree (coverage min(1, |A|) has kinks where a pixel's area
    crosses 1 or 0; a kink within h makes the difference at h no derivative)"""
    fd, fd2, ok = R.fd(par["ctrl"], par["colors"], par["widths"], target, g, idx, h=h, h2=h / 10)
    floor = 1e-3 * np.abs(fd).max()
    return fd, ok & (rel_err(fd2, fd, floor) < 2e-4), floor


def test_reference_adjoint_matches_finite_differences():
    R, par, target = _small()
    _, *grads = R.backward(par["ctrl"], par["colors"], par["widths"], target)
    g, idx = _sample(R, 48, np.random.default_rng(1))
    fd, ok, floor = smooth_fd(R, par, target, g, idx)
    an = _pick(grads, g, idx)
    assert ok.sum() >= 40
    assert rel_err(an[ok], fd[ok], floor).max() < 3e-4


def test_incremental_fd_equals_full_forward_fd():
    R, par, target = _small()
    g, idx = _sample(R, 12, np.random.default_rng(2))
    a, oka = R.fd(par["ctrl"], par["colors"], par["widths"], target, g, idx)
    b, okb = R.fd(par["ctrl"], par["colors"], par["widths"], target, g, idx, full=True)
    assert np.array_equal(oka, okb)
    assert np.abs(a - b).max() <= 1e-9 * np.abs(b).max()


def test_d_canvas_backward_is_the_loss_backward():
    """backward with d_canvas = dMSE/dcanvas equals the target form"""
    R, par, target = _small()
    canvas, loss = R.forward(par["ctrl"], par["colors"], par["widths"], target)
    l1, *g1 = R.backward(par["ctrl"], par["colors"], par["widths"], target)
    dc = 2 * (canvas - target) / canvas.size
    _, *g2 = R.backward(par["ctrl"], par["colors"], par["widths"], None, dc)
    assert abs(l1 - loss) < 1e-15
    for a, b in zip(g1, g2):
        assert np.abs(a - b).max() <= 1e-12 * max(np.abs(a).max(), 1e-30)


# ------------------------------------------------------------------ GPU


def _dev(a):
    import torch

    return torch.tensor(np.ascontiguousarray(a, np.float32), device="cuda")


def _host(t):
    return t.detach().cpu().numpy().astype(np.float64)


def _gpu_eval(gb, scene, par, target):
    A = gb.Analytic(scene)
    p = {k: _dev(v) for k, v in par.items()}
    t = _dev(target) if target is not None else None
    canvas, loss = A.forward(p["ctrl"], p["colors"], p["widths"], t)
    canvas = _host(canvas)
    loss = float(loss.item()) if loss is not None else None
    grads = A.backward() if target is not None else None
    assert A.sync() == 0
    out = canvas, loss, (tuple(_host(g) for g in grads) if grads else None), A
    return out


def _config3():
    scene, par = scenes.analytic_scene(seed=3)
    _, tpar = scenes.analytic_scene(seed=4)
    return scene, par, tpar


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["small", "config3"])
def test_gpu_flattening_bit_exact(gb, which):
    scene, par = scenes.analytic_scene(seed=3, n_paths=8, n_cubics=4, size=64) if which == "small" else \
        scenes.analytic_scene(seed=3)
    R = ar.Reference(scene)
    f32, _, seg = R.flatten(par["ctrl"])
    _, _, _, A = _gpu_eval(gb, scene, par, None)
    pts, off = A.points()
    assert np.array_equal(off, seg)
    assert np.array_equal(pts.view(np.uint32), f32.view(np.uint32))
    A.destroy()


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["small", "config3"])
def test_gpu_forward_and_gradient_match_fp64(gb, which):
    if which == "small":
        scene, par = scenes.analytic_scene(seed=3, n_paths=8, n_cubics=4, size=64)
        _, tpar = scenes.analytic_scene(seed=4, n_paths=8, n_cubics=4, size=64)
    else:
        scene, par, tpar = _config3()
    R = ar.Reference(scene)
    target, _ = R.forward(tpar["ctrl"], tpar["colors"], tpar["widths"])
    ref_canvas, ref_loss = R.forward(par["ctrl"], par["colors"], par["widths"], target)
    _, *ref = R.backward(par["ctrl"], par["colors"], par["widths"], target)
    _, _, _, _, ref_pts = R.backward(par["ctrl"], par["colors"], par["widths"], target, points=True)
    canvas, loss, grads, A = _gpu_eval(gb, scene, par, target)
    assert np.abs(canvas - ref_canvas).max() < CANVAS_TOL
    assert abs(loss - ref_loss) <= 1e-4 * ref_loss
    for name, a, b in zip(("ctrl", "colors", "widths", "points"), grads + (A.point_grads(),), ref + [ref_pts]):
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        scale = np.abs(b).max()
        per = np.abs(a - b) / np.maximum(np.abs(b), 1e-3 * scale)
        print("%s %s: rel L2 %.3g, per-parameter p99 %.3g max %.3g" % (which, name, err, np.quantile(per, 0.99),
                                                                       per.max()))
        assert err < GRAD_TOL, (name, err)
    A.destroy()


@pytest.mark.gpu
def test_gpu_gradient_matches_fp64_finite_differences(gb):
    """256 random parameters of the 256x256, 128-path scene (128 control
    coordinates, 64 colour components, 64 widths): GPU gradient vs FP64
    central differences, h = 1e-3.  Relative error |g - fd| / max(|fd|,
    1e-3 max|fd|); parameters whose flattening changes within h are not
    differentiable there and are replaced."""
    scene, par, tpar = _config3()
    R = ar.Reference(scene)
    target, _ = R.forward(tpar["ctrl"], tpar["colors"], tpar["widths"])
    _, _, grads, A = _gpu_eval(gb, scene, par, target)
    rng = np.random.default_rng(3)
    g, idx = _sample(R, 320, rng)
    fd, ok, floor = smooth_fd(R, par, target, g, idx)
    keep = np.zeros(len(g), bool)
    for grp, want in ((0, 128), (1, 64), (2, 64)):
        sel = np.nonzero((g == grp) & ok)[0][:want]
        assert len(sel) == want
        keep[sel] = True
    an = _pick(grads, g, idx)
    err = rel_err(an[keep], fd[keep], floor)
    print("analytic FD check: max rel err %.3g, median %.3g, %d of %d drawn not smooth at h" %
          (err.max(), np.median(err), int((~ok[:np.nonzero(keep)[0].max() + 1]).sum()),
           np.nonzero(keep)[0].max() + 1))
    assert err.max() < GRAD_TOL
    A.destroy()


class AnalyticRender:
    """torch.autograd.Function over the C-ABI forward / adjoint (test harness only)"""

    @staticmethod
    def make(gb, scene):
        import torch

        A = gb.Analytic(scene)

        class Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, ctrl, colors, widths):
                canvas, _ = A.forward(ctrl, colors, widths)
                return canvas.clone()

            @staticmethod
            def backward(ctx, d_canvas):
                return A.backward(d_canvas.contiguous())

        return Fn, A


@pytest.mark.gpu
def test_gpu_autograd_wrapper_matches_fused_loss(gb):
    import torch

    scene, par = scenes.analytic_scene(seed=3, n_paths=16, n_cubics=8, size=96)
    _, tpar = scenes.analytic_scene(seed=4, n_paths=16, n_cubics=8, size=96)
    R = ar.Reference(scene)
    target, _ = R.forward(tpar["ctrl"], tpar["colors"], tpar["widths"])
    Fn, A = AnalyticRender.make(gb, scene)
    p = {k: _dev(v).requires_grad_(True) for k, v in par.items()}
    t = _dev(target)
    canvas = Fn.apply(p["ctrl"], p["colors"], p["widths"])
    loss = torch.mean((canvas - t) ** 2)
    loss.backward()
    _, _, fused, A2 = _gpu_eval(gb, scene, par, target)
    for k, b in zip(("ctrl", "colors", "widths"), fused):
        a = _host(p[k].grad)
        assert np.abs(a - b).max() <= 1e-5 * np.abs(b).max() + 1e-12, k
    assert A.sync() == 0
    A.destroy(), A2.destroy()


@pytest.mark.gpu
def test_gpu_adam_steps_reduce_loss(gb):
    import torch

    scene, par = scenes.analytic_scene(seed=3, n_paths=32, n_cubics=8, size=128)
    _, tpar = scenes.analytic_scene(seed=4, n_paths=32, n_cubics=8, size=128)
    R = ar.Reference(scene)
    target = _dev(R.forward(tpar["ctrl"], tpar["colors"], tpar["widths"])[0])
    A = gb.Analytic(scene)
    p = {k: _dev(v) for k, v in par.items()}
    m = {k: torch.zeros_like(v) for k, v in p.items()}
    v = {k: torch.zeros_like(v) for k, v in p.items()}
    lr = {"ctrl": (0.5, -1e4, 1e4), "colors": (0.01, 0.0, 1.0), "widths": (0.05, 0.1, 16.0)}
    losses = []
    for step in range(1, 41):
        _, loss = A.forward(p["ctrl"], p["colors"], p["widths"], target)
        losses.append(loss.clone())
        grads = A.backward()
        for k, gk in zip(("ctrl", "colors", "widths"), grads):
            A.adam(p[k], gk, m[k], v[k], step, *lr[k])
    assert A.sync() == 0
    losses = [float(x.item()) for x in losses]
    assert losses[-1] < 0.8 * losses[0], losses
    A.destroy()


@pytest.mark.gpu
def test_gpu_ragged_and_degenerate_inputs(gb):
    """canvas sides that are no multiple of the band height, contours of one
    point and of lines only, repeated points, a path fully outside, huge and
    NaN control points: equal to the reference (NaN points are dropped on
    both sides; control points up to 1e5 px, where an fp32 edge still places
    its canvas crossing within the tolerance).  (A contour of zero area would sit on the kink of min(1, |A|)
    at 0, where the split of the gradient between coincident points is not
    defined; the repeated point here is in a contour with area.)"""
    kinds = [scenes.AN_LINE] * 4 + [scenes.AN_LINE] + [scenes.AN_CUBIC, scenes.AN_LINE] + [scenes.AN_CUBIC] * 2
    contours = [4, 1, 2, 2]
    ctrl = [(3, 4), (3, 4), (30.5, 20.25), (8, 26),   # repeated point
            (12, 12),                                  # a one-point contour
            (5, 30), (40, -20), (45, 60), (2, 25),     # cubic + line
            (-500, -500), (-400, -300), (-450, -420), (-300, -490), (-350, -350), (-420, -380)]  # outside
    sc = {"width": 37, "height": 29, "background": np.array([0.2, 0.1, 0.0, 0.5], np.float32),
          "path_ncontours": np.array([2, 1, 1], np.uint32),
          "path_flags": np.array([3, 3, 1], np.uint32),
          "contour_nseg": np.array(contours, np.uint32), "seg_kind": np.array(kinds, np.uint8)}
    par = {"ctrl": np.array(ctrl, np.float32), "colors": np.array([[0.3, 0.2, 0.1, 0.6], [0.1, 0.5, 0.2, 0.9],
                                                                    [0.0, 0.0, 0.7, 0.7]], np.float32),
           "widths": np.array([2.5, 1.0, 3.0], np.float32)}
    R = ar.Reference(sc)
    target = np.full((29, 37, 4), 0.5)
    for variant in ("plain", "huge", "nan"):
        q = {k: v.copy() for k, v in par.items()}
        if variant == "huge":
            q["ctrl"][6] = (1e5, -8e4)
        if variant == "nan":
            q["ctrl"][2] = (np.nan, 7.0)
        ref_canvas, ref_loss = R.forward(q["ctrl"], q["colors"], q["widths"], target)
        f32, _, seg = R.flatten(q["ctrl"])
        canvas, loss, grads, A = _gpu_eval(gb, sc, q, target)
        pts, off = A.points()
        assert np.array_equal(off, seg), variant
        assert np.array_equal(pts.view(np.uint32), f32.view(np.uint32)), variant
        assert np.abs(canvas - ref_canvas).max() < CANVAS_TOL, variant
        if variant == "plain":
            _, *ref = R.backward(q["ctrl"], q["colors"], q["widths"], target)
            for a, b in zip(grads, ref):
                assert np.abs(a - b).max() <= 1e-3 * np.abs(b).max() + 1e-9
        A.destroy()


@pytest.mark.gpu
def test_gpu_point_buffer_growth(gb):
    """a flattening that outgrows the point buffer: sync reports
    VKVG_STATUS_NO_MEMORY once, the buffer grows, the repeated call is exact"""
    scene, par = scenes.analytic_scene(seed=5, n_paths=2, n_cubics=32, size=64)
    R = ar.Reference(scene)
    A = gb.Analytic(scene)
    p = {k: _dev(v) for k, v in par.items()}
    A.forward(p["ctrl"], p["colors"], p["widths"])
    assert A.sync() == 0
    big = par["ctrl"].astype(np.float64) * 2e4 - 6.4e5
    pb = _dev(big)
    A.forward(pb, p["colors"], p["widths"])
    assert A.sync() == 1  # VKVG_STATUS_NO_MEMORY
    A.forward(pb, p["colors"], p["widths"])
    assert A.sync() == 0
    pts, off = A.points()
    f32, _, seg = R.flatten(big.astype(np.float32))
    assert len(pts) > 65536 and np.array_equal(off, seg)
    assert np.array_equal(pts.view(np.uint32), f32.view(np.uint32))
    A.destroy()


# ----------------------------------------------------- tiled evaluation


def test_quadratic_elevation_adjoint():
    """the glyph scene's quadratic outlines reach the analytic mode as exact
    cubic elevations; elevate_adjoint is elevate's transpose"""
    _, _, quad = scenes.analytic_glyph_scene(n_outlines=60, n_strokes=8, size=96)
    rng = np.random.default_rng(4)
    P, Q = rng.normal(size=quad["P"].shape), rng.normal(size=quad["Q"].shape)
    y = rng.normal(size=(3 * len(P), 2))
    lhs = np.sum(scenes.elevate(quad, P, Q).astype(np.float64) * y)
    gP, gQ = scenes.elevate_adjoint(quad, y)
    assert abs(lhs - (np.sum(P * gP) + np.sum(Q * gQ))) <= 1e-5 * abs(lhs)


def _gpu_eval_tiled(gb, scene, par, target, tile):
    A = gb.Analytic(scene, tile=tile)
    p = {k: _dev(v) for k, v in par.items()}
    canvas, loss = A.forward(p["ctrl"], p["colors"], p["widths"], _dev(target))
    canvas, loss = _host(canvas), float(loss.item())
    grads = tuple(_host(g) for g in A.backward())
    assert A.sync() == 0
    A.destroy()
    return canvas, loss, grads


@pytest.mark.gpu
@pytest.mark.parametrize("tile", [48, 128])
def test_gpu_tiled_matches_whole_canvas(gb, tile):
    """the tiled evaluation (tiles of 48 and 128 pixels, ragged at the canvas
    edge, paths crossing tiles and leaving the canvas) equals the
    whole-canvas one: canvas, loss and every gradient"""
    scene, par = scenes.analytic_scene(seed=3, n_paths=40, n_cubics=6, size=300, w_min=1.0, w_max=9.0)
    _, tpar = scenes.analytic_scene(seed=4, n_paths=40, n_cubics=6, size=300)
    par["ctrl"] = par["ctrl"] * np.float32(1.1) - np.float32(15.0)  # some control points off the canvas
    R = ar.Reference(scene)
    target, _ = R.forward(tpar["ctrl"], tpar["colors"], tpar["widths"])
    c0, l0, g0, A = _gpu_eval(gb, scene, par, target)
    A.destroy()
    c1, l1, g1 = _gpu_eval_tiled(gb, scene, par, target, tile)
    assert np.abs(c1 - c0).max() < 1e-5
    assert abs(l1 - l0) <= 1e-5 * l0
    for name, a, b in zip(("ctrl", "colors", "widths"), g1, g0):
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err < 1e-4, (name, err)


def _quad_fd(R, scene, quad, par, target, which, k, axis, h):
    """FP64 central difference of the loss in one outline coordinate (an
    on-curve point, which 0, or an off-curve one, which 1) through the
    quadratic elevation"""
    out = []
    for sgn in (1.0, -1.0):
        P, Q = quad["P"].astype(np.float64), quad["Q"].astype(np.float64)
        (P if which == 0 else Q)[k, axis] += sgn * h
        ctrl = scenes.elevate(quad, P, Q)  # float64 points: elevated in float64
        out.append(R.forward(ctrl, par["colors"], par["widths"], target)[1])
    return (out[0] - out[1]) / (2 * h)


@pytest.mark.gpu
def test_gpu_glyph_crop_outline_gradients_match_fd(gb):
    """the glyph construction on a 128 x 128 crop, tiled: the gradients of 24
    random outline coordinates (on-curve and off-curve points, through the
    quadratic elevation) against FP64 central differences at h = 1e-3 px,
    relative error |g - fd| / max(|fd|, 1e-3 max|fd|) within the analytic
    mode's bar; a coordinate whose differences at h and h/10 disagree (a
    flattening that changes within h: not differentiable there) is replaced
    by the next draw"""
    scene, par, quad = scenes.analytic_glyph_scene(n_outlines=200, n_strokes=20, size=128)
    tscene, tpar, _ = scenes.analytic_glyph_scene(seed=6, n_outlines=200, n_strokes=20, size=128)
    target, _ = ar.Reference(tscene).forward(tpar["ctrl"], tpar["colors"], tpar["widths"])
    R = ar.Reference(scene)
    _, _, (gc, _, _) = _gpu_eval_tiled(gb, scene, par, target, 64)
    gP, gQ = scenes.elevate_adjoint(quad, gc)
    rng = np.random.default_rng(7)
    n = len(quad["P"])
    rows = []
    while len(rows) < 24:
        which, k, axis = int(rng.integers(2)), int(rng.integers(n)), int(rng.integers(2))
        f1 = _quad_fd(R, scene, quad, par, target, which, k, axis, 1e-3)
        f2 = _quad_fd(R, scene, quad, par, target, which, k, axis, 1e-2)
        if abs(f1 - f2) > 2e-3 * max(abs(f1), 1e-9):
            continue  # not smooth within h
        rows.append(((gP if which == 0 else gQ)[k, axis], f1))
    an, fd = np.array(rows).T
    floor = 1e-3 * np.abs(fd).max()
    err = rel_err(an, fd, floor)
    print("glyph crop outline FD check: max rel err %.3g, median %.3g" % (err.max(), np.median(err)))
    assert err.max() < GRAD_TOL


@pytest.mark.gpu
def test_gpu_tiled_pairs_beyond_32_bits_report_no_memory(gb):
    """a tiled scene whose (tile, layer) entries reach 2^32 (65,536 tiles of
    16 px on a 4096 x 4096 canvas by 65,536 layers): the forward reports
    VKVG_STATUS_NO_MEMORY before sizing anything, and the scene stays usable
    for its status"""
    scene, par = scenes.analytic_scene(seed=9, n_paths=32768, n_cubics=1, size=4096)
    A = gb.Analytic(scene, tile=16)
    assert A.nlayers == 65536
    p = {k: _dev(v) for k, v in par.items()}
    with pytest.raises(gb.VkvgError, match="status 1"):
        A.forward(p["ctrl"], p["colors"], p["widths"])
    assert A.sync() == 1  # VKVG_STATUS_NO_MEMORY
    A.destroy()


@pytest.mark.gpu
def test_gpu_small_curves_flatten_bit_exact(gb):
    """scenes of small curves (the glyph construction: a few points per
    segment) flatten one lane per segment: the points, their order and the
    segment offsets equal the reference's flattening bit for bit, tiled or
    not"""
    scene, par, _ = scenes.analytic_glyph_scene(n_outlines=300, n_strokes=30, size=160)
    f32, _, seg = ar.Reference(scene).flatten(par["ctrl"])
    assert len(f32) <= 8 * len(scene["seg_kind"])  # the lane-per-segment case
    for tile in (0, 64):
        A = gb.Analytic(scene, tile=tile)
        p = {k: _dev(v) for k, v in par.items()}
        A.forward(p["ctrl"], p["colors"], p["widths"])
        A.forward(p["ctrl"], p["colors"], p["widths"])  # the second forward runs in the chosen mode
        assert A.sync() == 0
        pts, off = A.points()
        assert np.array_equal(off, seg)
        assert np.array_equal(pts.view(np.uint32), f32.view(np.uint32))
        A.destroy()


@pytest.mark.gpu
def test_gpu_tiled_glyph_crop_matches_fp64(gb):
    """the large glyph configuration's analytic construction on a 192 x 192
    crop at its density (440 quadratic outlines with holes, 44 closed
    strokes), tiled: canvas and loss against the FP64 reference, and the
    gradients of the outline control points (chained through the quadratic
    elevation) within the analytic mode's bar"""
    scene, par, quad = scenes.analytic_glyph_scene(n_outlines=440, n_strokes=44, size=192)
    # the target: another draw of the construction (its own structure)
    tscene, tpar, _ = scenes.analytic_glyph_scene(seed=6, n_outlines=440, n_strokes=44, size=192)
    target, _ = ar.Reference(tscene).forward(tpar["ctrl"], tpar["colors"], tpar["widths"])
    R = ar.Reference(scene)
    ref_canvas, ref_loss = R.forward(par["ctrl"], par["colors"], par["widths"], target)
    _, rc, rcol, rw = R.backward(par["ctrl"], par["colors"], par["widths"], target)
    canvas, loss, (gc, gcol, gw) = _gpu_eval_tiled(gb, scene, par, target, 64)
    assert np.abs(canvas - ref_canvas).max() < CANVAS_TOL
    assert abs(loss - ref_loss) <= 1e-4 * ref_loss
    gP, gQ = scenes.elevate_adjoint(quad, gc)
    rP, rQ = scenes.elevate_adjoint(quad, rc)
    for name, a, b in (("on-curve", gP, rP), ("off-curve", gQ, rQ), ("colors", gcol, rcol), ("widths", gw, rw)):
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err < GRAD_TOL, (name, err)
