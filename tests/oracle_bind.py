"""ctypes binding of the CPU oracle (oracle/libvko.so) for the tests and the
bench's CPU-baseline leg.  Test infrastructure: the product package never
imports this module."""
import ctypes as C
import os
import sys

import numpy as np

_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(_ROOT, "oracle"))
import build as _oracle_build  # noqa: E402

_lib = None


class Matrix(C.Structure):
    _fields_ = [("xx", C.c_float), ("yx", C.c_float), ("xy", C.c_float),
                ("yy", C.c_float), ("x0", C.c_float), ("y0", C.c_float)]


_F = C.c_float
_P = C.c_void_p
_U = C.c_uint32
_SIGS = {
    "vko_set_math_mode": (None, [C.c_int]),
    "vko_get_math_mode": (C.c_int, []),
    "vko_set_raster_mode": (None, [C.c_int]),
    "vko_set_threads": (None, [C.c_int]),
    "vko_pmath_eval": (None, [C.c_int, _P, _P, _P, C.c_uint64]),
    "vko_flatten_cubic": (_U, [_F, _P, _P, _U]),
    "vko_surface_create": (_P, [_U, _U, _U]),
    "vko_surface_destroy": (None, [_P]),
    "vko_surface_status": (C.c_int, [_P]),
    "vko_surface_clear": (None, [_P]),
    "vko_surface_write_to_memory": (C.c_int, [_P, _P]),
    "vko_surface_resolve_premult": (C.c_int, [_P, _P]),
    "vko_surface_read_samples": (C.c_int, [_P, _P]),
    "vko_surface_write_to_png": (C.c_int, [_P, C.c_char_p]),
    "vko_create": (_P, [_P]),
    "vko_destroy": (None, [_P]),
    "vko_status": (C.c_int, [_P]),
    "vko_flush": (None, [_P]),
    "vko_keep_draws": (None, [_P, C.c_int]),
    "vko_new_path": (None, [_P]),
    "vko_new_sub_path": (None, [_P]),
    "vko_close_path": (None, [_P]),
    "vko_move_to": (None, [_P, _F, _F]),
    "vko_rel_move_to": (None, [_P, _F, _F]),
    "vko_line_to": (None, [_P, _F, _F]),
    "vko_rel_line_to": (None, [_P, _F, _F]),
    "vko_curve_to": (None, [_P, _F, _F, _F, _F, _F, _F]),
    "vko_rel_curve_to": (None, [_P, _F, _F, _F, _F, _F, _F]),
    "vko_quadratic_to": (None, [_P, _F, _F, _F, _F]),
    "vko_rel_quadratic_to": (None, [_P, _F, _F, _F, _F]),
    "vko_arc": (None, [_P, _F, _F, _F, _F, _F]),
    "vko_arc_negative": (None, [_P, _F, _F, _F, _F, _F]),
    "vko_elliptic_arc_to": (None, [_P, _F, _F, C.c_bool, C.c_bool, _F, _F, _F]),
    "vko_rel_elliptic_arc_to": (None, [_P, _F, _F, C.c_bool, C.c_bool, _F, _F, _F]),
    "vko_ellipse": (None, [_P, _F, _F, _F, _F, _F]),
    "vko_rectangle": (C.c_int, [_P, _F, _F, _F, _F]),
    "vko_rounded_rectangle": (C.c_int, [_P, _F, _F, _F, _F, _F]),
    "vko_has_current_point": (C.c_bool, [_P]),
    "vko_get_current_point": (None, [_P, _P, _P]),
    "vko_path_extents": (None, [_P, _P, _P, _P, _P]),
    "vko_fill": (None, [_P]),
    "vko_fill_preserve": (None, [_P]),
    "vko_stroke": (None, [_P]),
    "vko_stroke_preserve": (None, [_P]),
    "vko_paint": (None, [_P]),
    "vko_clear": (None, [_P]),
    "vko_reset_clip": (None, [_P]),
    "vko_clip": (None, [_P]),
    "vko_clip_preserve": (None, [_P]),
    "vko_save": (None, [_P]),
    "vko_restore": (None, [_P]),
    "vko_set_source_rgba": (None, [_P, _F, _F, _F, _F]),
    "vko_set_source_rgb": (None, [_P, _F, _F, _F]),
    "vko_set_source_color": (None, [_P, _U]),
    "vko_pattern_create_linear": (_P, [_F, _F, _F, _F]),
    "vko_pattern_status": (C.c_int, [_P]),
    "vko_pattern_reference": (_P, [_P]),
    "vko_pattern_get_reference_count": (_U, [_P]),
    "vko_pattern_destroy": (None, [_P]),
    "vko_pattern_edit_linear": (C.c_int, [_P, _F, _F, _F, _F]),
    "vko_pattern_create_radial": (_P, [_F, _F, _F, _F, _F, _F]),
    "vko_pattern_create_for_surface": (_P, [_P]),
    "vko_pattern_set_extend": (None, [_P, C.c_int]),
    "vko_pattern_set_filter": (None, [_P, C.c_int]),
    "vko_set_source_surface": (None, [_P, _P, _F, _F]),
    "vko_pattern_edit_radial": (C.c_int, [_P, _F, _F, _F, _F, _F, _F]),
    "vko_pattern_add_color_stop": (C.c_int, [_P, _F, _F, _F, _F, _F]),
    "vko_pattern_get_color_stop_count": (C.c_int, [_P, _P]),
    "vko_pattern_set_matrix": (None, [_P, _P]),
    "vko_set_source": (None, [_P, _P]),
    "vko_set_line_width": (None, [_P, _F]),
    "vko_set_miter_limit": (None, [_P, _F]),
    "vko_set_line_cap": (None, [_P, C.c_int]),
    "vko_set_line_join": (None, [_P, C.c_int]),
    "vko_set_fill_rule": (None, [_P, C.c_int]),
    "vko_set_operator": (None, [_P, C.c_int]),
    "vko_set_opacity": (None, [_P, _F]),
    "vko_set_dash": (None, [_P, _P, _U, _F]),
    "vko_set_matrix": (None, [_P, _P]),
    "vko_get_matrix": (None, [_P, _P]),
    "vko_get_line_width": (_F, [_P]),
    "vko_get_line_join": (C.c_int, [_P]),
    "vko_get_line_cap": (C.c_int, [_P]),
    "vko_get_fill_rule": (C.c_int, [_P]),
    "vko_get_operator": (C.c_int, [_P]),
    "vko_identity_matrix": (None, [_P]),
    "vko_translate": (None, [_P, _F, _F]),
    "vko_scale": (None, [_P, _F, _F]),
    "vko_rotate": (None, [_P, _F]),
    "vko_transform": (None, [_P, _P]),
    "vko_get_color": (_U, [_P]),
    "vko_draw_count": (_U, [_P]),
    "vko_draw_info": (C.c_int, [_P, _U, _P]),
    "vko_draw_points": (C.c_int, [_P, _U, _P, _P]),
    "vko_draw_stroke": (C.c_int, [_P, _U, _P, _P]),
    "vko_draw_coverage": (C.c_int, [_P, _U, C.c_int, _P]),
    "vko_snap": (None, [_P, _U, _F, _F, _P, _P]),
    "vko_coverage_edges": (None, [_U, _U, _U, _P, C.c_uint64, _P]),
    "vko_matrix_init_identity": (None, [_P]),
    "vko_matrix_init": (None, [_P, _F, _F, _F, _F, _F, _F]),
    "vko_matrix_init_translate": (None, [_P, _F, _F]),
    "vko_matrix_init_scale": (None, [_P, _F, _F]),
    "vko_matrix_init_rotate": (None, [_P, _F]),
    "vko_matrix_translate": (None, [_P, _F, _F]),
    "vko_matrix_scale": (None, [_P, _F, _F]),
    "vko_matrix_rotate": (None, [_P, _F]),
    "vko_matrix_multiply": (None, [_P, _P, _P]),
    "vko_matrix_transform_distance": (None, [_P, _P, _P]),
    "vko_matrix_transform_point": (None, [_P, _P, _P]),
    "vko_matrix_invert": (C.c_int, [_P]),
    "vko_matrix_get_scale": (None, [_P, _P, _P]),
}


def lib():
    """Load (building first if needed) the oracle shared library."""
    global _lib
    if _lib is None:
        path = _oracle_build.build()
        _lib = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


def ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class OracleContext:
    """Thin object wrapper: attribute access maps `ctx.move_to(x, y)` to
    vko_move_to(ctx, x, y), mirroring the vkvg API."""

    def __init__(self, surf):
        self.L = lib()
        self.h = self.L.vko_create(surf)
        assert self.h

    def __getattr__(self, name):
        fn = getattr(self.L, "vko_" + name)
        return lambda *a: fn(self.h, *a)

    def set_dash(self, dashes, offset):
        arr = np.asarray(dashes, dtype=np.float32)
        self.L.vko_set_dash(self.h, ptr(arr) if len(arr) else None, len(arr), offset)

    def set_matrix(self, m):
        mm = Matrix(*m)
        self.L.vko_set_matrix(self.h, C.byref(mm))

    def set_source_linear(self, x0, y0, x1, y1, stops, pmat=None):
        """a linear gradient pattern as the source (created, used, released)"""
        p = self.L.vko_pattern_create_linear(x0, y0, x1, y1)
        for st in stops:
            self.L.vko_pattern_add_color_stop(p, *st)
        if pmat is not None:
            mm = Matrix(*pmat)
            self.L.vko_pattern_set_matrix(p, C.byref(mm))
        self.L.vko_set_source(self.h, p)
        self.L.vko_pattern_destroy(p)

    def set_source_surface(self, surf, x, y):
        self.L.vko_set_source_surface(self.h, surf.s, x, y)

    def set_source_surface_pattern(self, surf, extend, filt, pmat=None):
        """a surface pattern with sampler settings as the source"""
        p = self.L.vko_pattern_create_for_surface(surf.s)
        self.L.vko_pattern_set_extend(p, extend)
        self.L.vko_pattern_set_filter(p, filt)
        if pmat is not None:
            mm = Matrix(*pmat)
            self.L.vko_pattern_set_matrix(p, C.byref(mm))
        self.L.vko_set_source(self.h, p)
        self.L.vko_pattern_destroy(p)

    def set_source_radial(self, cx0, cy0, r0, cx1, cy1, r1, stops, pmat=None):
        """a radial gradient pattern as the source (created, used, released)"""
        p = self.L.vko_pattern_create_radial(cx0, cy0, r0, cx1, cy1, r1)
        for st in stops:
            self.L.vko_pattern_add_color_stop(p, *st)
        if pmat is not None:
            mm = Matrix(*pmat)
            self.L.vko_pattern_set_matrix(p, C.byref(mm))
        self.L.vko_set_source(self.h, p)
        self.L.vko_pattern_destroy(p)

    def current_point(self):
        x, y = C.c_float(), C.c_float()
        self.L.vko_get_current_point(self.h, C.byref(x), C.byref(y))
        return x.value, y.value

    def draws(self):
        """List of recorded draws with their geometry (needs keep_draws(1))."""
        out = []
        info = np.zeros(8, np.uint32)
        for i in range(self.L.vko_draw_count(self.h)):
            self.L.vko_draw_info(self.h, i, ptr(info))
            kind, npts, nsub, nverts, ninds, color, convex = [int(v) for v in info[:7]]
            d = {"kind": kind, "color": color, "convex": convex}
            if kind in (0, 1, 5, 6):
                pts = np.zeros((max(npts, 1), 2), np.float32)
                sub = np.zeros(max(nsub, 1), np.uint32)
                self.L.vko_draw_points(self.h, i, ptr(pts), ptr(sub))
                d["points"] = pts[:npts]
                d["subpaths"] = sub[:nsub]
            if kind == 2:
                v = np.zeros((max(nverts, 1), 2), np.float32)
                ix = np.zeros(max(ninds, 1), np.uint32)
                self.L.vko_draw_stroke(self.h, i, ptr(v), ptr(ix))
                d["verts"] = v[:nverts]
                d["inds"] = ix[:ninds]
            out.append(d)
        return out

    def coverage(self, i, w, h, samples, mode=0):
        out = np.zeros((h, w, samples), np.int32)
        self.L.vko_draw_coverage(self.h, i, mode, ptr(out))
        return out

    def destroy(self):
        if self.h:
            self.L.vko_destroy(self.h)
            self.h = None


class OracleSurface:
    def __init__(self, w, h, samples=4):
        self.L = lib()
        self.w, self.h, self.samples = w, h, samples
        self.s = self.L.vko_surface_create(w, h, samples)

    def image(self):
        out = np.zeros((self.h, self.w, 4), np.uint8)
        self.L.vko_surface_write_to_memory(self.s, ptr(out))
        return out

    def premult(self):
        out = np.zeros((self.h, self.w, 4), np.uint8)
        self.L.vko_surface_resolve_premult(self.s, ptr(out))
        return out

    def samples_rgba(self):
        out = np.zeros((self.h, self.w, self.samples, 4), np.uint8)
        self.L.vko_surface_read_samples(self.s, ptr(out))
        return out

    def context(self):
        return OracleContext(self.s)

    def destroy(self):
        if self.s:
            self.L.vko_surface_destroy(self.s)
            self.s = None


def pmath(fn, a, b=None):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(a if b is None else b, np.float32)
    out = np.empty_like(a)
    lib().vko_pmath_eval(fn, ptr(a), ptr(b), ptr(out), a.size)
    return out
