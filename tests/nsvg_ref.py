"""vkvg's vendored nanoSVG (src/nsvg/nanosvg.h), built from the reference tree
into oracle/_ref by oracle/build_ref.py, read through the dump interface of
oracle/nsvg_ref.c (test infrastructure only).  Only where the reference tree
is present: available() is False elsewhere (the GPU machine), and the tests that
need it skip.  parse() returns the same records as vkvg_gb300.Svg.shapes()."""
import ctypes as C
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import build_ref  # noqa: E402

_lib = None


def available():
    return build_ref.available()


def reference_dir():
    """the reference tree the recipe reads (VKVG_REFERENCE or its default)"""
    return build_ref.REFERENCE


def lib():
    global _lib
    if _lib is None:
        path = build_ref.build()
        if path is None:
            raise RuntimeError("the reference tree is absent: nanoSVG is not built")
        L = C.CDLL(path)
        P, U = C.c_void_p, C.c_uint32
        L.nref_parse.restype = P
        L.nref_parse.argtypes = [C.c_char_p, C.c_char_p, C.c_float]
        L.nref_free.argtypes = [P]
        L.nref_dims.argtypes = [P, P, P]
        L.nref_shape_count.restype = U
        L.nref_shape_count.argtypes = [P]
        L.nref_shape.argtypes = [P, U, P, P, P]
        L.nref_path.argtypes = [P, U, U, P, U, P, P]
        _lib = L
    return _lib


def parse(text, units=b"px", dpi=96.0):
    """(width, height, shapes) of nsvgParse(text, units, dpi)"""
    L = lib()
    h = L.nref_parse(text, units, dpi)
    if not h:
        raise RuntimeError("nsvgParse failed")
    w, hh = C.c_float(), C.c_float()
    L.nref_dims(h, C.byref(w), C.byref(hh))
    shapes = []
    for i in range(L.nref_shape_count(h)):
        idb = C.create_string_buffer(64)
        u = np.zeros(6, np.uint32)
        f = np.zeros(6, np.float32)
        L.nref_shape(h, i, idb, u.ctypes.data_as(C.c_void_p), f.ctypes.data_as(C.c_void_p))
        paths = []
        for p in range(int(u[5])):
            n, closed = C.c_uint32(), C.c_uint32()
            L.nref_path(h, i, p, None, 0, C.byref(n), C.byref(closed))
            pts = np.zeros((max(n.value, 1), 2), np.float32)
            L.nref_path(h, i, p, pts.ctypes.data_as(C.c_void_p), n.value, C.byref(n), C.byref(closed))
            paths.append((pts[:n.value], bool(closed.value)))
        shapes.append({"id": idb.value, "fill_type": int(u[0]), "fill_color": int(u[1]), "stroke_type": int(u[2]),
                       "stroke_color": int(u[3]), "visible": bool(u[4]), "opacity": f[0], "stroke_width": f[1],
                       "bounds": f[2:6].copy(), "paths": paths})
    L.nref_free(h)
    return np.float32(w.value), np.float32(hh.value), shapes
