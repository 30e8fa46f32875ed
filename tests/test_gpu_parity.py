"""GPU parity: every stage of the sm_103a pipeline against the CPU oracle on
the same seeded inputs, through the C ABI.

Bar: flattened points, stroke vertices and indices bit-exact (the kernels and
the oracle share the portable math and fp32 op order), per-sample winding /
covering-triangle counts bit-exact, and the final samples and image
bit-exact (integer UNORM8 blending on both sides)."""
import numpy as np
import pytest

import parity_util as pu
from vkvg_gb300 import scenes

pytestmark = pytest.mark.gpu


def small_scenes():
    out = [
        scenes.plain_small(n_polys=12, size=96, seed=0),
        scenes.curve_heavy(n_paths=10, size=128, seed=1, n_min=3, n_max=6),
        scenes.api_mix(n_items=24, size=160, seed=5),
        scenes.clip_mix(n_items=10, size=128, seed=13),
    ]
    for o in out:
        o["samples"] = 4
    return out


@pytest.mark.parametrize("fn", range(6))
def test_pmath_device_matches_host(gb, fn):
    rng = np.random.default_rng(100 + fn)
    a = rng.uniform(-50, 50, 100000).astype(np.float32)
    b = rng.uniform(-50, 50, 100000).astype(np.float32)
    if fn in (1, 4):
        a = rng.uniform(-1.1, 1.1, 100000).astype(np.float32)
    h = gb.pmath(fn, a, b, device=False)
    d = gb.pmath(fn, a, b, device=True)
    assert np.array_equal(h.view(np.uint32), d.view(np.uint32))


@pytest.mark.parametrize("idx", [0, 1, 2, 3])
def test_geometry_bit_exact(gb, vko, idx):
    sc = small_scenes()[idx]
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc)
    assert ctx.debug_counts()[5] == 0  # device status word
    errs = pu.compare_geometry(ctx, octx)
    assert not errs, errs[:10]


def _oracle_geometry_draws(octx):
    return [i for i, d in enumerate(octx.draws()) if d["kind"] < pu.STENCIL_OPS]


@pytest.mark.parametrize("idx", [0, 1, 2, 3])
def test_coverage_bit_exact(gb, vko, idx):
    sc = small_scenes()[idx]
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc)
    gi, oi = pu.geometry_draws(ctx), _oracle_geometry_draws(octx)
    assert len(gi) == len(oi)
    for i, j in zip(gi, oi):
        g = ctx.debug_coverage(i)
        o = octx.coverage(j, sc["width"], sc["height"], sc["samples"], mode=0)
        assert np.array_equal(g, o), "draw %d: %d samples differ" % (i, int((g != o).sum()))


@pytest.mark.parametrize("idx", [0, 1, 2, 3])
def test_image_bit_exact(gb, vko, idx):
    sc = small_scenes()[idx]
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc)
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    assert np.array_equal(surf.image(), osurf.image())


@pytest.mark.parametrize("idx", [0, 1, 2, 3])
def test_gpu_matches_golden(gb, idx):
    """the GPU library against the committed fixtures (tests/golden/), with no
    oracle run: image, per-draw kinds, fill points, stroke buffers and the
    digest of every draw's per-sample coverage"""
    import os
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_golden

    sc = small_scenes()[idx]
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", sc["name"] + ".npz"))
    dev, surf, ctx = pu.run_gpu(gb, sc)
    assert np.array_equal(surf.image(), g["image"])
    first, count, _ = ctx.debug_subpaths()
    gi = pu.geometry_draws(ctx)
    kinds = np.array([int(ctx.debug_draw(i)[0]) for i in gi], np.uint32)
    assert np.array_equal(kinds, g["kinds"])
    fp, sv, si = [], [], []
    for j, i in enumerate(gi):
        info = ctx.debug_draw(i)
        if kinds[j] in make_golden.FILL_KINDS:
            fp.append(pu.gpu_draw_points(ctx, info, first, count)[0])
        elif kinds[j] == 2:
            v, ix = ctx.debug_stroke(i)
            sv.append(v)
            si.append(ix)
        if kinds[j] in make_golden.FILL_KINDS + (2,):
            assert np.array_equal(make_golden.digest(ctx.debug_coverage(i)), g["cov_sha256"][j]), i
    for parts, key, dt in ((fp, "fill_pts", np.float32), (sv, "stroke_verts", np.float32), (si, "stroke_inds", np.uint32)):
        cat = np.concatenate(parts) if parts else np.zeros_like(g[key])
        assert np.array_equal(cat.astype(dt).view(np.uint32), g[key].view(np.uint32)), key


def _twice_dashed_scene():
    """the same paths stroked twice with different dash patterns
    (stroke_preserve then stroke): a subpath in two dashed stroke pairs"""
    r = scenes.SplitMix64(21)
    ops = [("set_source_rgb", 1.0, 1.0, 1.0), ("paint",)]
    for i in range(6):
        ops.append(("move_to", r.rnd() * 120, r.rnd() * 120))
        for _ in range(3):
            ops.append(("curve_to",) + tuple(r.rnd() * 120 for _ in range(6)))
        if i % 2:
            ops.append(("close_path",))
        ops += [("set_line_width", 1 + 5 * r.rnd()), ("set_line_cap", i % 3), ("set_line_join", (i + 1) % 3),
                ("set_dash", [6.0, 3.0], 1.5), ("set_source_rgba", 0.8, 0.1, 0.1, 0.6), ("stroke_preserve",),
                ("set_dash", [2.0, 4.0, 1.0], 0.0), ("set_source_rgba", 0.1, 0.1, 0.8, 0.5), ("stroke",)]
    return {"name": "twice_dashed", "width": 128, "height": 128, "samples": 4, "ops": ops, "paths": 6}


def test_twice_dashed_bit_exact(gb, vko):
    sc = _twice_dashed_scene()
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc)
    errs = pu.compare_geometry(ctx, octx)
    assert not errs, errs[:10]
    assert np.array_equal(surf.image(), osurf.image())


@pytest.mark.parametrize("w,h,samples", [(1300, 96, 4), (2100, 40, 4), (333, 77, 1), (17, 9, 4)])
def test_ragged_and_wide_surfaces_bit_exact(gb, vko, w, h, samples):
    """surfaces wider than one 1024-pixel raster tile (edges left of a tile,
    inside it and right of it), widths that are not multiples of 16, heights
    that end inside a band, and single-sample surfaces"""
    r = scenes.SplitMix64(w * 7 + h)
    ops = [("set_source_rgb", 1.0, 1.0, 1.0), ("paint",)]
    for i in range(14):
        ops.append(("move_to", r.rnd() * w * 1.2 - 0.1 * w, r.rnd() * h * 1.2 - 0.1 * h))
        for _ in range(3):
            ops.append(("curve_to",) + tuple(v for _ in range(3) for v in (r.rnd() * w * 1.2 - 0.1 * w,
                                                                           r.rnd() * h * 1.2 - 0.1 * h)))
        ops.append(("close_path",))
        ops += [("set_fill_rule", i % 2), ("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), 0.4 + 0.6 * r.rnd()),
                ("fill_preserve",), ("set_line_width", 1 + 6 * r.rnd()), ("set_line_join", i % 3),
                ("set_line_cap", i % 3), ("set_dash", [7.0, 4.0] if i % 3 == 0 else [], 0.0),
                ("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), 0.5 + 0.5 * r.rnd()), ("stroke",)]
    sc = {"name": "ragged", "width": w, "height": h, "samples": samples, "ops": ops, "paths": 14}
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc)
    assert ctx.debug_counts()[5] == 0
    errs = pu.compare_geometry(ctx, octx)
    assert not errs, errs[:10]
    n = int(ctx.debug_counts()[2])
    for i in range(n):
        if int(ctx.debug_draw(i)[0]) in (0, 1, 2):
            g = ctx.debug_coverage(i)
            o = octx.coverage(i, w, h, samples, mode=0)
            assert np.array_equal(g, o), "draw %d: %d samples differ" % (i, int((g != o).sum()))
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    assert np.array_equal(surf.image(), osurf.image())


def test_wide_surface_small_shapes_bit_exact(gb, vko):
    """a surface three raster tiles wide with shapes that lie inside one tile,
    straddle a tile boundary, or cover a whole tile with edges only outside
    it (left of the surface and right of the tile): the raster passes over
    the draws whose edges all lie left or all right of a tile"""
    w, h = 3000, 40
    r = scenes.SplitMix64(91)
    ops = [("set_source_rgb", 1.0, 1.0, 1.0), ("paint",),
           ("rectangle", -50.0, 4.0, 2950.0, 10.0), ("set_source_rgba", 0.2, 0.6, 0.3, 0.7), ("fill",),
           ("move_to", 900.0, 20.0), ("line_to", 2200.0, 22.0), ("line_to", 2150.0, 36.0), ("line_to", 950.0, 33.0),
           ("close_path",), ("set_source_rgba", 0.7, 0.2, 0.5, 0.6), ("fill_preserve",),
           ("set_line_width", 3.0), ("set_source_rgba", 0.1, 0.1, 0.1, 0.9), ("stroke",)]
    centres = [1024.0, 2048.0, 3.0, 2996.0] + [r.rnd() * w for _ in range(40)]
    for i, cx in enumerate(centres):
        cy = r.rnd() * h
        rad = 2.0 + 14.0 * r.rnd()
        ops.append(("move_to", cx + rad, cy))
        for k in range(1, 7):
            a = k * 2.0 * np.pi / 7
            ops.append(("line_to", cx + rad * np.cos(a) * (0.6 + 0.4 * r.rnd()), cy + rad * np.sin(a)))
        ops.append(("close_path",))
        ops += [("set_fill_rule", i % 2), ("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), 0.4 + 0.6 * r.rnd()),
                ("fill_preserve",), ("set_line_width", 1 + 4 * r.rnd()), ("set_line_join", i % 3),
                ("set_line_cap", i % 3), ("set_dash", [5.0, 3.0] if i % 4 == 0 else [], 0.0),
                ("set_source_rgba", r.rnd(), r.rnd(), r.rnd(), 0.5 + 0.5 * r.rnd()), ("stroke",)]
    sc = {"name": "wide_small", "width": w, "height": h, "samples": 4, "ops": ops, "paths": len(centres) + 2}
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc)
    assert ctx.debug_counts()[5] == 0
    errs = pu.compare_geometry(ctx, octx)
    assert not errs, errs[:10]
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    assert np.array_equal(surf.image(), osurf.image())


def test_empty_and_degenerate_paths(gb, vko):
    """fills and strokes of empty, single-point, zero-length and NaN paths
    draw nothing and leave no error; a degenerate-only frame still resolves"""
    nan = float("nan")
    ops = [("set_source_rgb", 0.2, 0.3, 0.4), ("paint",), ("fill",), ("stroke",),
           ("move_to", 10.0, 10.0), ("fill",), ("move_to", 10.0, 10.0), ("stroke",),
           ("move_to", 5.0, 5.0), ("line_to", 5.0, 5.0), ("line_to", 5.0, 5.0), ("stroke",),
           ("move_to", 5.0, 5.0), ("line_to", 5.0, 5.0), ("close_path",), ("fill",),
           ("move_to", nan, 3.0), ("line_to", 20.0, 20.0), ("line_to", 30.0, 5.0), ("fill_preserve",), ("stroke",),
           ("move_to", 8.0, 8.0), ("curve_to", 8.0, 8.0, 8.0, 8.0, 8.0, 8.0), ("stroke",),
           ("set_line_width", 0.0), ("move_to", 1.0, 1.0), ("line_to", 30.0, 30.0), ("stroke",)]
    sc = {"name": "degenerate", "width": 40, "height": 40, "samples": 4, "ops": ops, "paths": 0}
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc)
    assert ctx.debug_counts()[5] == 0
    assert not pu.compare_geometry(ctx, octx)
    assert np.array_equal(surf.image(), osurf.image())


@pytest.mark.parametrize("samples,radial", [(4, False), (1, False), (4, True), (1, True)])
def test_gradient_sources_bit_exact(gb, vko, samples, radial):
    """linear and radial gradient sources (more distinct gradients than one
    frame holds, so the recording is flushed in between): samples and image
    equal the oracle's"""
    sc = scenes.gradient_mix(n_items=14, size=144, seed=9, samples=samples, radial=radial)
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc)
    assert ctx.debug_counts()[5] == 0
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    assert np.array_equal(surf.image(), osurf.image())


def test_curve_heavy_full_size_bit_exact(gb, vko):
    """The full 1024x1024, 2,048-path benchmark scene: every stroke/fill draw's
    geometry and the final 4x MSAA samples equal the oracle's."""
    import os

    sc = scenes.curve_heavy()
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc, threads=os.cpu_count() or 1)
    assert ctx.debug_counts()[5] == 0
    errs = pu.compare_geometry(ctx, octx)
    assert not errs, errs[:10]
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    assert np.array_equal(surf.image(), osurf.image())


@pytest.mark.parametrize("name", [s["name"] for s in scenes.vkvg_clip_cases()])
def test_vkvg_clip_cases_bit_exact(gb, vko, name):
    """vkvg's clip and save/restore demo sequences (tests/clip.c,
    tests/save_restore.c) at 1024x800: samples and image equal the oracle's"""
    sc = [s for s in scenes.vkvg_clip_cases() if s["name"] == name][0]
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc, threads=8)
    assert ctx.debug_counts()[5] == 0 and ctx.status() == 0
    assert not pu.compare_geometry(ctx, octx)
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    assert np.array_equal(surf.image(), osurf.image())


@pytest.mark.parametrize("name", [s["name"] for s in scenes.vkvg_demo_cases()])
def test_vkvg_demo_cases_bit_exact(gb, vko, name):
    """vkvg's single-sequence demo programs (tests/line_caps.c, stroke.c,
    fill.c, fill_non_zero.c, dashes.c, line_join.c, circles.c, arcs.c,
    curve.c, colinear.c, fill_and_stroke.c, simple_paint.c, compositing.c,
    radial_gradient.c, gradient.c, rect_fill.c, transform.c, bezier.c,
    gradient2.c, inverse_colinear.c) at the
    harness's 512x512: geometry,
    samples and image equal the oracle's"""
    sc = [s for s in scenes.vkvg_demo_cases() if s["name"] == name][0]
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc, threads=8)
    assert ctx.debug_counts()[5] == 0 and ctx.status() == 0
    if ("flush",) not in sc["ops"]:  # the captured draws are the last frame's
        assert not pu.compare_geometry(ctx, octx)
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    assert np.array_equal(surf.image(), osurf.image())


@pytest.mark.parametrize("samples,flush_every", [(1, 0), (4, 2), (1, 3)])
def test_clip_mix_variants_bit_exact(gb, vko, samples, flush_every):
    """the clip scene at one sample, and flushed every few items so the clip
    planes, save planes and stencil images cross frames"""
    sc = scenes.clip_mix(n_items=10, size=120, seed=17, samples=samples, flush_every=flush_every)
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc)
    assert ctx.debug_counts()[5] == 0 and ctx.status() == 0
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    assert np.array_equal(surf.image(), osurf.image())


def test_clip_state_on_gpu(gb):
    """restore's state and statuses through the library: line join back to
    miter, INVALID_RESTORE without a save, a new context on a clipped surface
    starting unclipped"""
    dev = gb.Device(samples=4)
    surf = gb.Surface(dev, 32, 32)
    ctx = surf.context()
    ctx.set_line_width(3.0)
    ctx.set_line_join(1)
    ctx.save()
    ctx.set_line_width(9.0)
    ctx.restore()
    assert ctx.get_line_width() == 3.0 and ctx.get_line_join() == 0 and ctx.status() == 0
    ctx.rectangle(4.0, 4.0, 8.0, 8.0)
    ctx.clip()
    ctx.flush()
    ctx.destroy()
    ctx2 = surf.context()
    ctx2.set_source_rgb(0.0, 1.0, 0.0)
    ctx2.paint()
    ctx2.flush()
    assert (surf.image()[..., 1] == 255).all()  # the new context's stencil is clear
    ctx2.restore()
    assert ctx2.status() == 3  # VKVG_STATUS_INVALID_RESTORE


@pytest.mark.parametrize("which", ["api_mix", "clip_mix"])
def test_replay_stream_matches_calls(gb, vko, which):
    """vkvg_gb300_replay_stream of a scene's command codes gives the same
    samples as the scene's calls, and both equal the oracle's samples for
    those calls (vkvg's replay, src/recording/vkvg_record_internal.c:249,
    dispatches each code to the public call it records)"""
    import ctypes as C

    sc = scenes.api_mix(n_items=24, size=160, seed=5) if which == "api_mix" else \
        scenes.clip_mix(n_items=10, size=128, seed=13)
    sc["ops"] = [op for op in sc["ops"] if op[0] in scenes.CMD]  # vkvg records no opacity or pattern calls
    dev, surf, ctx = pu.run_gpu(gb, sc, debug=False)
    cmds, args = scenes.encode(sc["ops"])
    dev2 = gb.Device(samples=sc["samples"])
    surf2 = gb.Surface(dev2, sc["width"], sc["height"])
    ctx2 = surf2.context()
    st = ctx2.L.vkvg_gb300_replay_stream(ctx2.h, cmds.ctypes.data_as(C.c_void_p), len(cmds),
                                         args.ctypes.data_as(C.c_void_p), len(args))
    assert st == 0
    ctx2.flush()
    assert np.array_equal(surf.samples_rgba(), surf2.samples_rgba())
    osurf, octx = pu.run_oracle(vko, sc)
    assert np.array_equal(surf2.samples_rgba(), osurf.samples_rgba())
    assert np.array_equal(surf2.image(), osurf.image())


def test_radial_gradient_paint_bit_exact(gb, vko):
    """one radial gradient painted over a non-square surface, focus inside
    and focus pulled in by edit_radial, with a pattern matrix: the image
    equals the oracle's"""
    for args, pmat in (((60.0, 50.0, 5.0, 80.0, 64.0, 60.0), None),
                       ((140.0, 10.0, 3.0, 70.0, 60.0, 40.0), (1.1, 0.1, -0.2, 0.9, 4.0, -3.0))):
        stops = [(0.0, 1.0, 1.0, 0.0, 1.0), (0.5, 0.0, 0.5, 1.0, 0.8), (1.0, 0.2, 0.0, 0.4, 1.0)]
        ops = [("translate", 3.0, 2.0), ("set_source_radial",) + args + (stops, pmat), ("paint",)]
        sc = {"name": "radial_paint", "width": 160, "height": 128, "samples": 4, "ops": ops, "paths": 0}
        dev, surf, ctx = pu.run_gpu(gb, sc)
        osurf, octx = pu.run_oracle(vko, sc)
        assert ctx.status() == 0 and ctx.debug_counts()[5] == 0
        assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())


@pytest.mark.parametrize("samples", [4, 1])
def test_surface_sources_bit_exact(gb, vko, samples):
    """surface sources (offsets, every extend mode, nearest and bilinear,
    pattern matrices, opacity, save / restore, the offset a gradient leaves
    behind): samples and image equal the oracle's"""
    sc = scenes.surface_mix(n_items=12, size=128, seed=23, samples=samples)
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc)
    assert ctx.status() == 0 and ctx.debug_counts()[5] == 0
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    assert np.array_equal(surf.image(), osurf.image())


def test_surface_source_outlives_its_handles(gb, vko):
    """a surface used as a source and destroyed by the caller before the
    frame runs stays valid for that frame; the pattern holds a reference"""
    dev = gb.Device(samples=4)
    src = gb.Surface(dev, 20, 12)
    c = src.context()
    c.set_source_rgba(0.2, 0.6, 0.9, 0.8)
    c.paint()
    c.flush()
    c.destroy()
    L = gb.lib()
    before = L.vkvg_surface_get_reference_count(src.h)
    p = L.vkvg_pattern_create_for_surface(src.h)
    assert L.vkvg_surface_get_reference_count(src.h) == before + 1
    L.vkvg_pattern_destroy(p)
    assert L.vkvg_surface_get_reference_count(src.h) == before
    dst = gb.Surface(dev, 40, 30)
    ctx = dst.context()
    ctx.set_source_surface(src, 3.0, 2.0)
    ctx.rectangle(0.0, 0.0, 30.0, 20.0)
    ctx.fill()
    ctx.set_source_rgb(0.0, 0.0, 0.0)  # releases the pattern
    src.destroy()  # the caller's reference
    ctx.flush()
    assert ctx.status() == 0
    img = dst.premult()
    assert tuple(img[5, 10]) != (0, 0, 0, 0) and tuple(img[25, 35]) == (0, 0, 0, 0)


def _batch_case(gb, dev, sc):
    """a surface drawn by its own captured frame (executed once), and a
    second surface for the same frame in a batch"""
    import ctypes as C

    L = gb.lib()
    a = gb.Surface(dev, sc["width"], sc["height"])
    b = gb.Surface(dev, sc["width"], sc["height"])
    ctx = a.context()
    if "cmds" in sc:
        assert L.vkvg_gb300_replay_stream(ctx.h, sc["cmds"].ctypes.data_as(C.c_void_p), len(sc["cmds"]),
                                          sc["args"].ctypes.data_as(C.c_void_p), len(sc["args"])) == 0
    else:
        scenes.play(ctx, sc["ops"])
    fr = L.vkvg_gb300_frame_capture(ctx.h)
    assert fr
    assert L.vkvg_gb300_frame_execute(fr, a.h) == 0
    return a, b, ctx, fr


def test_batch_matches_frames(gb):
    """a batch of frames (curves, dashes, elliptic arcs and ellipses, uneven
    generated surfaces) leaves every surface as its own frame does, on the
    sizing run, on each tuning run and on graph replays"""
    import ctypes as C

    L = gb.lib()
    dev = gb.Device(samples=4)
    scs = [scenes.api_mix(n_items=24, size=160, seed=5), scenes.curve_heavy(n_paths=30, size=256, seed=4, n_min=3,
                                                                             n_max=10),
           scenes.plain_small(n_polys=12, size=96, seed=0)]
    scs += scenes.batch_streams(seed=2, n_surfaces=4, max_paths=80, min_paths=10, max_segs=40, max_side=1200)
    cases = [_batch_case(gb, dev, sc) for sc in scs]
    frames = (C.c_void_p * len(cases))(*[c[3] for c in cases])
    targets = (C.c_void_p * len(cases))(*[c[1].h for c in cases])
    bt = L.vkvg_gb300_batch_create(frames, targets, len(cases))
    assert bt
    t = np.zeros(9, np.float32)
    for run in range(17):  # sizing, fourteen tuning runs, graph capture and a replay
        assert L.vkvg_gb300_batch_execute(bt) == 0, run
        L.vkvg_gb300_batch_timing(bt, t.ctypes.data_as(C.c_void_p))
        for k, (a, b, _, _) in enumerate(cases):
            assert np.array_equal(a.samples_rgba(), b.samples_rgba()), (run, k)
            assert np.array_equal(a.image(), b.image()), (run, k)
    assert t[1] == 1 and t[6] == 1 and t[5] == len(cases)  # graph replay, tuned
    L.vkvg_gb300_batch_destroy(bt)
    for _, _, ctx, fr in cases:
        L.vkvg_gb300_frame_destroy(fr)
        ctx.destroy()


def test_batch_gradient_sources(gb, vko):
    """frames with pattern sources in a batch (linear and radial gradients,
    several per frame, a glyph crop under one gradient, and a frame without
    any): every surface equals its own frame's result and the oracle's, on
    the sizing run, tuning runs over every tile form and graph replays"""
    import ctypes as C

    L = gb.lib()
    dev = gb.Device(samples=4)
    scs = [scenes.gradient_mix(n_items=6, size=144, seed=9, samples=4),
           scenes.gradient_mix(n_items=5, size=200, seed=3, samples=4, radial=True),
           scenes.glyph_scene(n_outlines=200, n_strokes=20, size=160),
           scenes.curve_heavy(n_paths=8, size=120, seed=4, n_min=3, n_max=6)]
    cases = [_batch_case(gb, dev, sc) for sc in scs]
    frames = (C.c_void_p * len(cases))(*[c[3] for c in cases])
    targets = (C.c_void_p * len(cases))(*[c[1].h for c in cases])
    bt = L.vkvg_gb300_batch_create(frames, targets, len(cases))
    assert bt
    oracle = [pu.run_oracle(vko, sc)[0] for sc in scs]
    t = np.zeros(9, np.float32)
    for run in range(17):
        assert L.vkvg_gb300_batch_execute(bt) == 0, run
        L.vkvg_gb300_batch_timing(bt, t.ctypes.data_as(C.c_void_p))
        for k, (a, b, _, _) in enumerate(cases):
            assert np.array_equal(a.samples_rgba(), b.samples_rgba()), (run, k)
            if run in (0, 16):
                assert np.array_equal(b.samples_rgba(), oracle[k].samples_rgba()), (run, k)
                assert np.array_equal(b.image(), oracle[k].image()), (run, k)
    assert t[1] == 1 and t[6] == 1
    L.vkvg_gb300_batch_destroy(bt)
    for _, _, ctx, fr in cases:
        L.vkvg_gb300_frame_destroy(fr)
        ctx.destroy()


def test_batch_rejects_clip_and_duplicates(gb):
    import ctypes as C

    L = gb.lib()
    dev = gb.Device(samples=4)
    sc = {"name": "clipped", "width": 64, "height": 64, "samples": 4, "paths": 1,
          "ops": [("rectangle", 4.0, 4.0, 30.0, 30.0), ("clip",), ("set_source_rgb", 1.0, 0.0, 0.0), ("paint",)]}
    a, b, ctx, fr = _batch_case(gb, dev, sc)
    assert not L.vkvg_gb300_batch_create((C.c_void_p * 1)(fr), (C.c_void_p * 1)(b.h), 1)
    sc2 = scenes.plain_small(n_polys=4, size=64, seed=1)
    a2, b2, ctx2, fr2 = _batch_case(gb, dev, sc2)
    assert not L.vkvg_gb300_batch_create((C.c_void_p * 2)(fr2, fr2), (C.c_void_p * 2)(b2.h, b2.h), 2)
    for c, f in ((ctx, fr), (ctx2, fr2)):
        L.vkvg_gb300_frame_destroy(f)
        c.destroy()


@pytest.mark.gpu
@pytest.mark.parametrize("size,n,m", [(192, 300, 30), (256, 600, 60)])
def test_glyph_scene_bit_exact(gb, vko, size, n, m):
    """the large glyph scene's construction on a crop: quadratic outlines with
    holes (NON_ZERO), round-join strokes, one linear gradient source; samples
    bit-exact against the oracle"""
    sc = scenes.glyph_scene(n_outlines=n, n_strokes=m, size=size)
    dev, surf, ctx = pu.run_gpu(gb, sc, debug=False)
    osurf, octx = pu.run_oracle(vko, sc)
    assert ctx.status() == 0
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    assert np.array_equal(surf.image(), osurf.image())


def test_small_polygon_config_bit_exact(gb, vko):
    """The small polygon configuration as stated: 512x512 at 4x MSAA, 64
    closed polygons of 3-32 vertices uniform over the surface (seed 0,
    self-intersecting), each filled NON_ZERO in an opaque random colour and
    stroked in black at width 4, miter join (limit 10), butt cap.  Flattened
    points, stroke buffers, every draw's per-sample winding / covering counts,
    the samples and the image equal the oracle's."""
    sc = scenes.plain_small()
    assert (sc["width"], sc["height"], sc["paths"]) == (512, 512, 64)
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc, threads=8)
    assert ctx.debug_counts()[5] == 0 and ctx.status() == 0
    errs = pu.compare_geometry(ctx, octx)
    assert not errs, errs[:10]
    gi, oi = pu.geometry_draws(ctx), _oracle_geometry_draws(octx)
    assert len(gi) == len(oi) == 129  # the paint, 64 fills, 64 strokes
    for i, j in zip(gi, oi):
        g = ctx.debug_coverage(i)
        o = octx.coverage(j, sc["width"], sc["height"], sc["samples"], mode=0)
        assert np.array_equal(g, o), "draw %d: %d samples differ" % (i, int((g != o).sum()))
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    assert np.array_equal(surf.image(), osurf.image())


def test_batch_streams_match_oracle(gb, vko):
    """The uneven batch's own content through the batch: four generated
    surfaces (sides up to 512 so the oracle stays quick; cubics, lines and
    arcs of radius up to 200 px, path boxes log-uniform from 4 px, fill only,
    fill then stroke and stroke only, widths up to 12 px) rendered by one
    batch execution and by its graph replays; every surface's samples and
    image equal the oracle's rendering of the same command stream."""
    import ctypes as C

    L = gb.lib()
    dev = gb.Device(samples=4)
    scs = scenes.batch_streams(seed=2, n_surfaces=4, max_paths=240, min_paths=60, max_segs=400, max_side=512)
    ops_all = []
    for sc in scs:
        sc["samples"] = 4
        sc["ops"] = scenes.decode(sc["cmds"], sc["args"])
        ops_all += [op[0] for op in sc["ops"]]
    for name in ("curve_to", "line_to", "arc", "fill", "fill_preserve", "stroke"):
        assert name in ops_all, name
    cases = [_batch_case(gb, dev, sc) for sc in scs]
    frames = (C.c_void_p * len(cases))(*[c[3] for c in cases])
    targets = (C.c_void_p * len(cases))(*[c[1].h for c in cases])
    bt = L.vkvg_gb300_batch_create(frames, targets, len(cases))
    assert bt
    oracle = [pu.run_oracle(vko, sc, threads=8)[0] for sc in scs]
    for run in range(17):  # sizing, tuning runs, graph capture and a replay
        assert L.vkvg_gb300_batch_execute(bt) == 0, run
        if run in (0, 5, 11, 14, 16):
            for k, (a, b, _, _) in enumerate(cases):
                assert np.array_equal(b.samples_rgba(), oracle[k].samples_rgba()), (run, k)
                assert np.array_equal(b.image(), oracle[k].image()), (run, k)
    L.vkvg_gb300_batch_destroy(bt)
    for _, _, ctx, fr in cases:
        L.vkvg_gb300_frame_destroy(fr)
        ctx.destroy()


@pytest.fixture
def raster_form(gb):
    """sets the process-wide raster form for one test, then restores automatic"""
    L = gb.lib()
    yield lambda f: L.vkvg_gb300_debug_set_raster_form(f)
    L.vkvg_gb300_debug_set_raster_form(-1)


def _form_scenes():
    out = [scenes.curve_heavy(n_paths=12, size=200, seed=3, n_min=3, n_max=8),
           scenes.api_mix(n_items=24, size=160, seed=5),
           scenes.gradient_mix(n_items=14, size=144, seed=9, samples=4),
           scenes.gradient_mix(n_items=6, size=96, seed=2, samples=1, radial=True),
           scenes.surface_mix(n_items=8, size=112, seed=23, samples=4),
           scenes.glyph_scene(n_outlines=60, n_strokes=8, size=128)]
    for o in out:
        o.setdefault("samples", 4)
    wide = scenes.curve_heavy(n_paths=8, size=100, seed=6, n_min=3, n_max=6)
    wide["width"], wide["name"] = 1300, "wide1300"  # two tiles, the second ragged
    out.append(wide)
    return out


@pytest.mark.parametrize("form", [0, 1, 2, 3, 4, 5])
def test_each_raster_form_bit_exact(gb, vko, raster_form, form):
    """every raster form (the register tiles of 1024, 256, 128 and 64 pixels
    and the row form in half and whole bands) on solid, gradient (one source image and several), radial,
    surface-source and glyph scenes, one and four samples, a surface two
    tiles wide: the form asked for is the one that ran, and its samples and
    image equal the oracle's"""
    raster_form(form)
    for sc in _form_scenes():
        dev, surf, ctx = pu.run_gpu(gb, sc, debug=False)
        assert ctx.raster_form() == form, sc["name"]
        assert ctx.status() == 0 and ctx.debug_counts()[5] == 0, sc["name"]
        osurf, octx = pu.run_oracle(vko, sc)
        assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba()), sc["name"]
        assert np.array_equal(surf.image(), osurf.image()), sc["name"]


@pytest.mark.parametrize("form", [0, 3, 4])
def test_coverage_each_form_bit_exact(gb, vko, raster_form, form):
    """per-draw winding and covering counts read back through the row form and
    the wide register tile equal the oracle's"""
    raster_form(form)
    sc = scenes.curve_heavy(n_paths=10, size=128, seed=1, n_min=3, n_max=6)
    dev, surf, ctx = pu.run_gpu(gb, sc)
    osurf, octx = pu.run_oracle(vko, sc)
    assert ctx.raster_form() == form
    gi, oi = pu.geometry_draws(ctx), _oracle_geometry_draws(octx)
    for i, j in zip(gi, oi):
        g = ctx.debug_coverage(i)
        o = octx.coverage(j, sc["width"], sc["height"], sc["samples"], mode=0)
        assert np.array_equal(g, o), "draw %d: %d samples differ" % (i, int((g != o).sum()))


def test_contexts_on_several_threads(gb):
    """contexts on four host threads at once, one thread-aware device (each
    context flushes on its own stream, each surface has its own lock): every
    surface equals the same scene rendered alone, over three flushes each"""
    import threading

    scs = [scenes.api_mix(n_items=24, size=160, seed=40 + k) for k in range(4)]
    alone = [pu.run_gpu(gb, sc, debug=False)[1].image().copy() for sc in scs]
    dev = gb.Device(samples=4, thread_aware=True)
    out, errs = [[] for _ in scs], []

    def work(k):
        try:
            sc = scs[k]
            for _ in range(3):
                surf = gb.Surface(dev, sc["width"], sc["height"])
                ctx = surf.context()
                scenes.play(ctx, sc["ops"])
                ctx.flush()
                assert ctx.status() == 0
                out[k].append(surf.image().copy())
                ctx.destroy()
        except Exception as e:  # reported on the main thread
            errs.append((k, e))

    threads = [threading.Thread(target=work, args=(k,)) for k in range(len(scs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errs, errs
    for k in range(len(scs)):
        assert len(out[k]) == 3
        for img in out[k]:
            assert np.array_equal(img, alone[k]), k
