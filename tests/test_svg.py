"""SVG ingestion (include/vkvg-svg.h over vkvg_gb300/csrc/svg.cpp).

Parser parity: what vkvg's SVG walk reads from a parsed document (size, and
per shape id, paints, visibility, opacity, stroke width, bounds and the cubic
points of every path) is bit-identical to vkvg's own parser, nanoSVG
(src/nsvg/nanosvg.h): against committed fixtures of nanoSVG's output
everywhere, and against nanoSVG itself (built from the reference tree into
oracle/_ref) on the reference's SVG files and on seeded, quirky and mutated
documents where that tree is present.  Render parity (-m gpu):
vkvg_svg_render on the GPU equals the oracle driven through the same walk
(tests/svg_render.py) sample for sample."""
import ctypes as C
import glob
import os
import random

import numpy as np
import pytest

import nsvg_ref
import svg_render
from vkvg_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF_FILES = sorted(glob.glob("/root/reference/tests/data/*.svg") + glob.glob("/root/reference/doc/*.svg") +
                   glob.glob("/root/reference/doc/images/*.svg"))
needs_ref = pytest.mark.skipif(not nsvg_ref.available(), reason="the reference tree (nanoSVG) is absent")


def _golden():
    import sys

    sys.path.insert(0, GOLDEN)
    import make_svg_golden

    return make_svg_golden


@pytest.fixture(scope="module")
def gbl():
    import vkvg_gb300

    vkvg_gb300._build.build()
    return vkvg_gb300


def _parse(gbl, text):
    doc = gbl.Svg(text)
    try:
        return doc.dimensions(), doc.shapes()
    finally:
        doc.destroy()


def _same_shapes(a, b):
    """exact equality of two shape-record lists; returns the first mismatch"""
    if len(a) != len(b):
        return "shape count %d vs %d" % (len(a), len(b))
    for i, (x, y) in enumerate(zip(a, b)):
        for k in ("id", "fill_type", "fill_color", "stroke_type", "stroke_color", "visible"):
            if x[k] != y[k]:
                return "shape %d %s: %r vs %r" % (i, k, x[k], y[k])
        for k in ("opacity", "stroke_width", "bounds"):
            if not np.array_equal(np.float32(x[k]).view(np.uint32), np.float32(y[k]).view(np.uint32)):
                return "shape %d %s: %r vs %r" % (i, k, x[k], y[k])
        if len(x["paths"]) != len(y["paths"]):
            return "shape %d path count" % i
        for j, ((p, c), (q, d)) in enumerate(zip(x["paths"], y["paths"])):
            if c != d or p.shape != q.shape or not np.array_equal(p.view(np.uint32), q.view(np.uint32)):
                return "shape %d path %d differs" % (i, j)
    return None


@pytest.mark.parametrize("name", ["seed1", "seed2", "seed3", "seed4", "quirks5", "quirks6"])
def test_parser_matches_nanosvg_fixtures(gbl, name):
    mg = _golden()
    text = dict(mg.documents())[name]
    g = np.load(os.path.join(GOLDEN, "svg_%s.npz" % name))
    (w, h), shapes = _parse(gbl, text)
    assert (w, h) == (int(g["size"][0]), int(g["size"][1]))
    mine = mg.pack(g["size"][0], g["size"][1], shapes)
    for k in g.files:
        assert np.array_equal(mine[k], g[k]), (name, k)


@needs_ref
@pytest.mark.parametrize("path", REF_FILES, ids=lambda p: os.path.basename(p))
def test_parser_matches_nanosvg_on_reference_documents(gbl, path):
    text = open(path, "rb").read()
    rw, rh, ref = nsvg_ref.parse(text)
    (w, h), mine = _parse(gbl, text)
    assert (w, h) == (int(rw), int(rh))
    err = _same_shapes(ref, mine)
    assert err is None, err


@needs_ref
def test_parser_matches_nanosvg_on_seeded_and_mutated_documents(gbl):
    rnd = random.Random(11)
    docs = [scenes.svg_document(seed=s, n_shapes=25) for s in range(40)]
    docs += [scenes.svg_document(seed=100 + s, n_shapes=25, quirks=True) for s in range(40)]
    for s in range(40):
        d = bytearray(scenes.svg_document(seed=200 + s, n_shapes=15))
        for _ in range(rnd.randint(1, 4)):
            k = rnd.randint(0, 2)
            idx = [i for i, c in enumerate(d) if c == ord(">" if k == 0 else '"')]
            i = rnd.choice(idx)
            if k == 2:
                del d[i]
            else:
                d[i:i] = b" " * (k + 1)
        docs.append(bytes(d))
    for n, text in enumerate(docs):
        rw, rh, ref = nsvg_ref.parse(text)
        (w, h), mine = _parse(gbl, text)
        assert (w, h) == (int(rw), int(rh)), n
        err = _same_shapes(ref, mine)
        assert err is None, (n, err)


def test_svg_load_api(gbl, tmp_path):
    """vkvg_svg_load of a file and of a missing file, dimensions, and the
    document API's null handling"""
    L = gbl.lib()
    text = scenes.svg_document(seed=3, n_shapes=10)
    f = tmp_path / "doc.svg"
    f.write_bytes(text)
    h = L.vkvg_svg_load(str(f).encode())
    assert h
    w, hh = C.c_uint32(), C.c_uint32()
    L.vkvg_svg_get_dimensions(h, C.byref(w), C.byref(hh))
    assert (w.value, hh.value) == _parse(gbl, text)[0]
    assert L.vkvg_gb300_svg_shape_count(h) == len(_parse(gbl, text)[1])
    L.vkvg_svg_destroy(h)
    assert not L.vkvg_svg_load(str(tmp_path / "missing.svg").encode())
    L.vkvg_svg_destroy(None)
    assert L.vkvg_gb300_svg_shape_count(None) == 0


# ------------------------------------------------------------------ GPU


@pytest.mark.gpu
@pytest.mark.parametrize("name,samples", [("seed1", 4), ("quirks5", 4), ("seed2", 1)])
def test_svg_render_bit_exact(gb, vko, name, samples):
    """vkvg_svg_render of a parsed document equals the oracle driven through
    vkvg's walk over the same shapes"""
    text = dict(_golden().documents())[name]
    doc = gb.Svg(text)
    (w, h), shapes = doc.dimensions(), doc.shapes()
    dev = gb.Device(samples=samples)
    surf = gb.Surface(dev, w, h)
    ctx = surf.context()
    ctx.set_source_rgb(1.0, 1.0, 1.0)
    ctx.paint()
    doc.render(ctx)
    ctx.flush()
    assert ctx.status() == 0
    osurf = vko.OracleSurface(w, h, samples)
    octx = osurf.context()
    octx.set_source_rgb(1.0, 1.0, 1.0)
    octx.paint()
    svg_render.render(octx, shapes)
    octx.flush()
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    doc.destroy()


@pytest.mark.gpu
def test_svg_render_subset_and_surface_from_fragment(gb, vko):
    """render limited to one id (a group's id reaches its shapes), and
    vkvg_surface_create_from_svg_fragment: the document's size, drawn at the
    device's dpi"""
    text = dict(_golden().documents())["seed3"]
    doc = gb.Svg(text)
    (w, h), shapes = doc.dimensions(), doc.shapes()
    ids = [s["id"] for s in shapes if s["id"]]
    sub = max(set(ids), key=ids.count)
    dev = gb.Device(samples=4)
    surf = gb.Surface(dev, w, h)
    ctx = surf.context()
    doc.render(ctx, sub)
    ctx.flush()
    osurf = vko.OracleSurface(w, h, 4)
    octx = osurf.context()
    svg_render.render(octx, shapes, sub)
    octx.flush()
    assert np.array_equal(surf.samples_rgba(), osurf.samples_rgba())
    L = gb.lib()
    L.vkvg_device_set_dpy(dev.h, 96, 96)  # the dpi vkvg_svg_load_fragment parses at
    s2 = L.vkvg_surface_create_from_svg_fragment(dev.h, 0, 0, text)
    assert s2 and L.vkvg_surface_status(s2) == 0
    assert (L.vkvg_surface_get_width(s2), L.vkvg_surface_get_height(s2)) == (w, h)
    img = np.zeros((h, w, 4), np.uint8)
    assert L.vkvg_surface_write_to_memory(s2, img.ctypes.data_as(C.c_void_p)) == 0
    o2 = vko.OracleSurface(w, h, 4)
    c2 = o2.context()
    svg_render.render(c2, shapes)
    c2.flush()
    assert np.array_equal(img, o2.image())
    L.vkvg_surface_destroy(s2)
    doc.destroy()
