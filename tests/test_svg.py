"""SVG ingestion (include/vkvg-svg.h over vkvg_gb300/csrc/svg.cpp).

Parser parity: what vkvg's SVG walk reads from a parsed document
(src/nsvg/vkvg_nsvg.c:82-136: the size, and per shape its id, paints,
visibility, opacity, stroke width and the cubic points of every subpath)
against vkvg's own parser, nanoSVG (src/nsvg/nanosvg.h): the structure (shape
and subpath counts, point counts, closed flags, ids, paint kinds and colours)
identical, coordinates, stroke widths and opacities within 1e-3 px (the
vertex tolerance of the drop-in).  Against committed fixtures of nanoSVG's
output everywhere, and against nanoSVG itself (built from the reference tree
into oracle/_ref) on the reference's SVG files and on seeded documents where
that tree is present.  The reader's own grammar (numbers, arcs, entities,
comments, transforms, viewBox) is tested on hand-written documents.  Render
parity (-m gpu): vkvg_svg_render on the GPU equals the oracle driven through
the same walk (tests/svg_render.py) sample for sample."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

import nsvg_ref
import svg_render
from vkvg_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REFERENCE = nsvg_ref.reference_dir()  # the reference tree, where present (oracle/build_ref.py)
REF_FILES = sorted(glob.glob(os.path.join(REFERENCE, "tests", "data", "*.svg")) +
                   glob.glob(os.path.join(REFERENCE, "doc", "*.svg")) +
                   glob.glob(os.path.join(REFERENCE, "doc", "images", "*.svg")))
needs_ref = pytest.mark.skipif(not nsvg_ref.available(), reason="the reference tree (nanoSVG) is absent")
TOL = 1e-3  # px


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


def _compare(ref, mine):
    """None if the shape lists agree (structure exactly, numbers within
    TOL), else the first difference; also the largest coordinate difference"""
    worst = 0.0
    if len(ref) != len(mine):
        return "shape count %d vs %d" % (len(ref), len(mine)), worst
    for i, (x, y) in enumerate(zip(ref, mine)):
        for k in ("id", "fill_type", "fill_color", "stroke_type", "stroke_color", "visible"):
            if x[k] != y[k]:
                return "shape %d %s: %r vs %r" % (i, k, x[k], y[k]), worst
        for k in ("opacity", "stroke_width"):
            if abs(float(x[k]) - float(y[k])) > TOL:
                return "shape %d %s: %r vs %r" % (i, k, x[k], y[k]), worst
        if np.abs(np.float64(x["bounds"]) - y["bounds"]).max() > TOL:
            return "shape %d bounds: %r vs %r" % (i, x["bounds"], y["bounds"]), worst
        if len(x["paths"]) != len(y["paths"]):
            return "shape %d subpath count %d vs %d" % (i, len(x["paths"]), len(y["paths"])), worst
        for j, ((p, c), (q, d)) in enumerate(zip(x["paths"], y["paths"])):
            if c != d or p.shape != q.shape:
                return "shape %d subpath %d: %s %s vs %s %s" % (i, j, p.shape, c, q.shape, d), worst
            e = float(np.abs(np.float64(p) - q).max()) if p.size else 0.0
            worst = max(worst, e)
            if e > TOL:
                return "shape %d subpath %d: coordinates differ by %g" % (i, j, e), worst
    return None, worst


@pytest.mark.parametrize("name", ["seed1", "seed2", "seed3", "seed4", "quirks5", "quirks6"])
def test_parser_matches_nanosvg_fixtures(gbl, name):
    mg = _golden()
    text = dict(mg.documents())[name]
    g = np.load(os.path.join(GOLDEN, "svg_%s.npz" % name))
    (w, h), mine = _parse(gbl, text)
    assert (w, h) == (int(g["size"][0]), int(g["size"][1]))
    err, worst = _compare(mg.unpack(g), mine)
    assert err is None, (name, err)
    assert worst <= TOL


@needs_ref
@pytest.mark.parametrize("path", REF_FILES, ids=lambda p: os.path.basename(p))
def test_parser_matches_nanosvg_on_reference_documents(gbl, path):
    text = open(path, "rb").read()
    rw, rh, ref = nsvg_ref.parse(text)
    (w, h), mine = _parse(gbl, text)
    assert (w, h) == (int(rw), int(rh))
    err, _ = _compare(ref, mine)
    assert err is None, err


@needs_ref
def test_parser_matches_nanosvg_on_seeded_documents(gbl):
    docs = [scenes.svg_document(seed=s, n_shapes=25) for s in range(40)]
    docs += [scenes.svg_document(seed=100 + s, n_shapes=25, quirks=True) for s in range(40)]
    total = same = 0
    for n, text in enumerate(docs):
        rw, rh, ref = nsvg_ref.parse(text)
        (w, h), mine = _parse(gbl, text)
        assert (w, h) == (int(rw), int(rh)), n
        err, _ = _compare(ref, mine)
        assert err is None, (n, err)
        for x, y in zip(ref, mine):
            for (p, _), (q, _) in zip(x["paths"], y["paths"]):
                total += p.size
                same += int(np.sum(p.view(np.uint32) == q.view(np.uint32)))
    assert same > 0.9 * total  # most coordinates are bit-identical as well


@pytest.mark.parametrize("name", ["seed1", "seed2", "seed3", "seed4", "quirks5", "quirks6"])
def test_render_of_reader_parse_equals_render_of_nanosvg_parse(gbl, vko, name):
    """vkvg's walk over this reader's shapes and over nanoSVG's (the
    fixtures), both rendered by the oracle at 4x MSAA: the same image, byte
    for byte (the GPU equals the oracle on the reader's shapes,
    test_svg_render_bit_exact)"""
    mg = _golden()
    text = dict(mg.documents())[name]
    g = np.load(os.path.join(GOLDEN, "svg_%s.npz" % name))
    (w, h), mine = _parse(gbl, text)
    imgs = []
    for shapes in (mg.unpack(g), mine):
        o = vko.OracleSurface(w, h, 4)
        c = o.context()
        c.set_source_rgb(1.0, 1.0, 1.0)
        c.paint()
        svg_render.render(c, shapes)
        c.flush()
        imgs.append(o.image())
    assert np.array_equal(imgs[0], imgs[1])


def _one(gbl, body, size='width="100" height="100"'):
    (w, h), shapes = _parse(gbl, ('<svg %s>%s</svg>' % (size, body)).encode())
    return (w, h), shapes


def test_reader_number_and_path_grammar(gbl):
    """SVG 1.1 path data: implicit lineto after moveto, numbers packed
    without separators (".5.5", "-1-2", exponents), exponent versus an em
    unit, relative commands, arc flags packed without separators"""
    _, s = _one(gbl, '<path d="M10,20l.5.5-1-2 1e1,0 1.5E+1-1e-1"/>')
    p = s[0]["paths"][0][0]
    assert np.allclose(p[[0, 3, 6, 9, 12]], [[10, 20], [10.5, 20.5], [9.5, 18.5], [19.5, 18.5], [34.5, 18.4]],
                       atol=1e-5)
    _, s = _one(gbl, '<path d="M0 0 H10 V10 h-5 v-5 z" font-size="3" stroke-width="2em"/>'
                     '<path d="M0 0 H10" stroke-width="2em" font-size="3"/>')
    assert s[0]["paths"][0][1] and len(s[0]["paths"][0][0]) == 1 + 3 * 5
    assert s[0]["stroke_width"] == 6.0 and s[1]["stroke_width"] == 0.0  # em: the font-size read so far
    _, a = _one(gbl, '<path d="M10 50 A40 40 0 0110 49.99 M0 0 a5 5 0 1 0 10 0"/>')
    _, b = _one(gbl, '<path d="M10 50 A40 40 0 0 1 10 49.99 M0 0 a5 5 0 1 0 10 0"/>')
    assert len(a[0]["paths"]) == 2
    for (p, _), (q, _) in zip(a[0]["paths"], b[0]["paths"]):
        assert np.array_equal(p, q)


def test_reader_smooth_curves_and_shapes(gbl):
    """S reflects the previous control point, T the previous quadratic one
    (a quadratic is its exact cubic); circle, rounded rect and polygon"""
    _, s = _one(gbl, '<path d="M0 0 C10 0 20 10 20 20 S30 40 40 40 Q50 40 50 50 T60 60"/>')
    p = s[0]["paths"][0][0]
    assert np.allclose(p[4], [20, 30])  # 2 (20, 20) - (20, 10)
    q = np.float32([50, 40])
    assert np.allclose(p[7], np.float32([40, 40]) + np.float32(2 / 3) * (q - np.float32([40, 40])), atol=1e-5)
    t = 2 * np.float32([50, 50]) - q  # reflected quadratic control point
    assert np.allclose(p[10], np.float32([50, 50]) + np.float32(2 / 3) * (t - np.float32([50, 50])), atol=1e-5)
    _, s = _one(gbl, '<circle cx="50" cy="50" r="10"/><rect x="1" y="2" width="30" height="20" rx="4"/>'
                     '<polygon points="0,0 10,0 10,10"/>')
    c = s[0]["paths"][0][0]
    assert len(c) == 1 + 3 * 5 and np.allclose(c[0], [60, 50]) and np.allclose(c[3], [50, 60])  # + closing line
    r = s[1]["paths"][0][0]
    assert len(r) == 1 + 3 * 9 and np.allclose(r[0], [5, 2])  # 4 edges, 4 corners, the closing line
    g = s[2]["paths"][0]
    assert g[1] and len(g[0]) == 1 + 3 * 3 and np.allclose(g[0][-1], [0, 0])


def test_reader_xml_and_style(gbl):
    """comments (holding tags), processing instructions, CDATA and entities;
    style declarations; transform lists applied right to left; colours"""
    body = ('<!-- <rect width="50" height="50"/> --><?pi x?><![CDATA[<rect/>]]>'
            '<g transform="translate(10 0) scale(2)" style="fill: #0f0; stroke:rgb(100%,0%,50%) ;opacity:.5">'
            '<path id="a&amp;b" d="M1 1 L2 1 L2 2Z"/></g>'
            '<path d="M0 0L1 0L1 1z" fill="orange" fill-opacity="0.5"/>')
    _, s = _one(gbl, body)
    assert len(s) == 2
    assert s[0]["id"] == b"a&b"
    assert np.allclose(s[0]["paths"][0][0][0], [12, 2])
    assert s[0]["fill_color"] == 0xff00ff00 and s[0]["stroke_color"] == (0xff << 24 | 127 << 16 | 255)
    assert abs(s[0]["opacity"] - 0.5) < 1e-7 and abs(s[0]["stroke_width"] - 2.0) < 1e-6
    assert s[1]["fill_color"] == (127 << 24 | 0x808080)  # a name vkvg's build does not know: grey


def test_reader_viewbox_and_start_tag_spacing(gbl):
    """viewBox with preserveAspectRatio meet / slice and their alignment;
    whitespace before a start tag's '>' is read as XML defines it (vkvg's
    parser reads on into the following tags there: outside the parity
    comparison)"""
    for par, x0 in (("xMidYMid meet", 25.0), ("xMinYMin meet", 0.0), ("xMaxYMax meet", 50.0)):
        (w, h), s = _one(gbl, '<path d="M0 0 L10 0 L10 10 Z"/>',
                         'width="100" height="50" viewBox="0 0 10 10" preserveAspectRatio="%s"' % par)
        assert (w, h) == (100, 50)
        assert np.allclose(s[0]["paths"][0][0][0], [x0, 0]) and abs(s[0]["stroke_width"] - 5.0) < 1e-6
    (w, h), s = _one(gbl, '<path d="M0 0 L10 0 L10 10 Z"/>', 'width="100" height="50" viewBox="0 0 10 10"')
    assert np.allclose(s[0]["paths"][0][0][6], [100, 50])  # none: scaled to fill
    _, s = _one(gbl, '<g id="a" ><rect width="5" height="5" ></rect></g><rect width="5" height="5"/>')
    assert [x["id"] for x in s] == [b"a", b""]


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
    assert L.vkvg_gb300_svg_shape(h, 10 ** 6, None, None, None) == -1
    L.vkvg_svg_destroy(h)
    assert not L.vkvg_svg_load(str(tmp_path / "missing.svg").encode())
    assert not L.vkvg_svg_load_fragment(None)
    L.vkvg_svg_destroy(None)
    L.vkvg_svg_render(None, None, None)
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
