"""vkvg_surface_write_to_png (src/vkvg_surface.c:283-391): the file the
library writes is decoded here independently (PNG signature and chunk
layout, every chunk's CRC-32, IHDR fields, the zlib stream inflated by
Python's zlib, which also checks its Adler-32, and the row filters) and its
pixels must equal vkvg_surface_write_to_memory's, which are the oracle's
(unpremultiplied RGBA8, vkvg's truncating conversion)."""
import os
import struct
import threading
import zlib

import numpy as np
import pytest

import parity_util as pu
from vkvg_gb300 import scenes

pytestmark = pytest.mark.gpu


def decode_png(path):
    """(width, height, RGBA8 array) of an 8-bit RGBA PNG with filter 0 rows;
    raises on a bad signature, chunk CRC or zlib stream"""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, []
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF, typ
        chunks.append((typ, body))
        pos += 12 + n
    assert pos == len(data)
    assert chunks[0][0] == b"IHDR" and chunks[-1] == (b"IEND", b"")
    w, h, depth, ctype, comp, filt, lace = struct.unpack(">IIBBBBB", chunks[0][1])
    assert (depth, ctype, comp, filt, lace) == (8, 6, 0, 0, 0)
    raw = zlib.decompress(b"".join(b for t, b in chunks if t == b"IDAT"))
    assert len(raw) == h * (1 + 4 * w)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 4 * w)
    assert (rows[:, 0] == 0).all()  # filter type none
    return w, h, rows[:, 1:].reshape(h, w, 4).copy()


@pytest.mark.parametrize("w,h", [(160, 144), (333, 77), (1, 1), (600, 230)])
def test_write_to_png_decodes_to_memory_image(gb, vko, tmp_path, w, h):
    """a scene with translucent colours (unpremultiplied by the write), ragged
    sizes, and an image larger than one 65,535-byte stored deflate block"""
    sc = scenes.api_mix(n_items=20, size=max(w, h), seed=5)
    sc["width"], sc["height"] = w, h
    dev, surf, ctx = pu.run_gpu(gb, sc, debug=False)
    path = str(tmp_path / "out.png")
    assert surf.write_png(path) == 0
    pw, ph, px = decode_png(path)
    assert (pw, ph) == (w, h)
    assert np.array_equal(px, surf.image())
    osurf, _ = pu.run_oracle(vko, sc)
    assert np.array_equal(px, osurf.image())


def test_write_to_png_concurrent_writers(gb, tmp_path):
    """host threads writing PNGs of different surfaces at once produce valid
    files (the CRC table is shared, read-only)"""
    dev = gb.Device(samples=4)
    surfs = []
    for k in range(4):
        s = gb.Surface(dev, 97 + 13 * k, 61 + 7 * k)
        c = s.context()
        c.set_source_rgba(0.1 * k, 0.5, 0.9 - 0.2 * k, 0.5 + 0.1 * k)
        c.paint()
        c.flush()
        c.destroy()
        surfs.append(s)
    want = [s.image() for s in surfs]
    errs = []

    def work(k):
        try:
            for rep in range(5):
                p = str(tmp_path / ("t%d_%d.png" % (k, rep)))
                assert surfs[k].write_png(p) == 0
                _, _, px = decode_png(p)
                assert np.array_equal(px, want[k])
        except Exception as e:  # reported below
            errs.append(e)

    th = [threading.Thread(target=work, args=(k,)) for k in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errs, errs


def test_write_to_png_bad_path(gb, tmp_path):
    """a path that cannot be opened gives VKVG_STATUS_WRITE_ERROR"""
    dev = gb.Device(samples=1)
    s = gb.Surface(dev, 8, 8)
    assert s.write_png(os.path.join(str(tmp_path), "missing_dir", "x.png")) == 8  # VKVG_STATUS_WRITE_ERROR
