"""Run one scene through the GPU library and the CPU oracle and collect the
per-stage results for comparison (test infrastructure)."""
import numpy as np

from vkvg_gb300 import scenes


def _gpu_sources(gb, dev, sc):
    out = []
    for s in sc.get("sources", ()):
        surf = gb.Surface(dev, s["width"], s["height"])
        c = surf.context()
        scenes.play(c, s["ops"])
        c.flush()
        c.destroy()
        out.append(surf)
    return out


def run_gpu(gb, sc, debug=True):
    dev = gb.Device(samples=sc["samples"])
    srcs = _gpu_sources(gb, dev, sc)
    surf = gb.Surface(dev, sc["width"], sc["height"])
    ctx = surf.context()
    if debug:
        ctx.debug_capture(True)
    scenes.play(ctx, sc["ops"], srcs)
    ctx.flush()
    surf.sources = srcs
    return dev, surf, ctx


def run_oracle(vko, sc, raster_mode=0, threads=1):
    L = vko.lib()
    L.vko_set_raster_mode(raster_mode)
    L.vko_set_threads(threads)
    srcs = []
    for s in sc.get("sources", ()):
        ss = vko.OracleSurface(s["width"], s["height"], sc["samples"])
        c = ss.context()
        scenes.play(c, s["ops"])
        c.flush()
        c.destroy()
        srcs.append(ss)
    surf = vko.OracleSurface(sc["width"], sc["height"], sc["samples"])
    ctx = surf.context()
    ctx.keep_draws(1)
    scenes.play(ctx, sc["ops"], srcs)
    ctx.flush()
    surf.sources = srcs
    return surf, ctx


def gpu_draw_points(ctx, info, first, count):
    """points of the subpaths a GPU draw references, and their counts"""
    xy, fl = ctx.debug_points()
    s0, ns = int(info[1]), int(info[2])
    cnt = count[s0:s0 + ns]
    pts = [xy[first[s]:first[s] + count[s]] for s in range(s0, s0 + ns)]
    return (np.concatenate(pts) if pts else np.zeros((0, 2), np.float32)), cnt


# draw kinds below this one carry geometry or colour (fills, strokes, paint,
# clear, clip paths); the stencil operations of reset_clip / save / restore
# above it may split differently between the library and the oracle
STENCIL_OPS = 7


def geometry_draws(gctx):
    """indices of the GPU context's draws that are not stencil operations"""
    n = int(gctx.debug_counts()[2])
    return [i for i in range(n) if int(gctx.debug_draw(i)[0]) < STENCIL_OPS]


def compare_geometry(gctx, octx):
    """bit-exact comparison of flattened points and stroke buffers per draw;
    returns a list of mismatch descriptions"""
    errs = []
    odraws = [d for d in octx.draws() if d["kind"] < STENCIL_OPS]
    first, count, flags = gctx.debug_subpaths()
    gidx = geometry_draws(gctx)
    if len(gidx) != len(odraws):
        return ["draw count %d vs oracle %d" % (len(gidx), len(odraws))]
    for gi, od in zip(gidx, odraws):
        i = gi
        info = gctx.debug_draw(i)
        if int(info[0]) != od["kind"]:
            errs.append("draw %d kind %d vs %d" % (i, info[0], od["kind"]))
            continue
        if od["kind"] in (0, 1, 5, 6):
            pts, cnt = gpu_draw_points(gctx, info, first, count)
            if not np.array_equal(cnt, od["subpaths"]):
                errs.append("draw %d subpath counts differ" % i)
            elif not np.array_equal(pts.view(np.uint32), od["points"].view(np.uint32)):
                d = np.abs(pts - od["points"]).max()
                errs.append("draw %d points differ (max %.3g)" % (i, d))
        elif od["kind"] == 2:
            v, ix = gctx.debug_stroke(i)
            if v.shape != od["verts"].shape or ix.shape != od["inds"].shape:
                errs.append("draw %d stroke sizes %s/%s vs %s/%s" % (i, v.shape, ix.shape, od["verts"].shape,
                                                                      od["inds"].shape))
            elif not np.array_equal(ix, od["inds"]):
                errs.append("draw %d stroke indices differ" % i)
            elif not np.array_equal(v.view(np.uint32), od["verts"].view(np.uint32)):
                errs.append("draw %d stroke vertices differ (max %.3g)" % (i, np.abs(v - od["verts"]).max()))
    return errs
