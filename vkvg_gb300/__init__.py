"""GB300-native implementation of vkvg's path hot path.

The product is the C-ABI shared library ``_build/libvkvg_gb300.so`` (declared
in include/vkvg.h and include/vkvg_gb300.h).  This module loads it with
ctypes and exposes thin object wrappers whose method names are vkvg's own
(``ctx.move_to(x, y)`` calls ``vkvg_move_to(ctx, x, y)``).  There is no
Python or CPU fallback: if the library is missing or no CUDA device is
present, loading or device creation raises.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB
_lib = None

_F, _P, _U, _I, _B = C.c_float, C.c_void_p, C.c_uint32, C.c_int, C.c_bool

# name -> (restype, argtypes); every vkvg_public function of include/*.h
SIGNATURES = {
    "vkvg_matrix_init_identity": (None, [_P]),
    "vkvg_matrix_init": (None, [_P, _F, _F, _F, _F, _F, _F]),
    "vkvg_matrix_init_translate": (None, [_P, _F, _F]),
    "vkvg_matrix_init_scale": (None, [_P, _F, _F]),
    "vkvg_matrix_init_rotate": (None, [_P, _F]),
    "vkvg_matrix_translate": (None, [_P, _F, _F]),
    "vkvg_matrix_scale": (None, [_P, _F, _F]),
    "vkvg_matrix_rotate": (None, [_P, _F]),
    "vkvg_matrix_multiply": (None, [_P, _P, _P]),
    "vkvg_matrix_transform_distance": (None, [_P, _P, _P]),
    "vkvg_matrix_transform_point": (None, [_P, _P, _P]),
    "vkvg_matrix_invert": (_I, [_P]),
    "vkvg_matrix_get_scale": (None, [_P, _P, _P]),
    "vkvg_device_create": (_P, [_P]),
    "vkvg_device_destroy": (None, [_P]),
    "vkvg_device_status": (_I, [_P]),
    "vkvg_device_reference": (_P, [_P]),
    "vkvg_device_get_reference_count": (_U, [_P]),
    "vkvg_device_set_dpy": (None, [_P, _I, _I]),
    "vkvg_device_get_dpy": (None, [_P, _P, _P]),
    "vkvg_device_set_context_cache_size": (None, [_P, _U]),
    "vkvg_surface_create": (_P, [_P, _U, _U]),
    "vkvg_surface_create_from_bitmap": (_P, [_P, _P, _U, _U]),
    "vkvg_surface_status": (_I, [_P]),
    "vkvg_surface_reference": (_P, [_P]),
    "vkvg_surface_get_reference_count": (_U, [_P]),
    "vkvg_surface_destroy": (None, [_P]),
    "vkvg_surface_clear": (None, [_P]),
    "vkvg_surface_get_width": (_U, [_P]),
    "vkvg_surface_get_height": (_U, [_P]),
    "vkvg_surface_write_to_png": (_I, [_P, C.c_char_p]),
    "vkvg_surface_write_to_memory": (_I, [_P, _P]),
    "vkvg_surface_resolve": (None, [_P]),
    "vkvg_create": (_P, [_P]),
    "vkvg_destroy": (None, [_P]),
    "vkvg_status": (_I, [_P]),
    "vkvg_status_to_string": (C.c_char_p, [_I]),
    "vkvg_reference": (_P, [_P]),
    "vkvg_get_reference_count": (_U, [_P]),
    "vkvg_flush": (None, [_P]),
    "vkvg_new_path": (None, [_P]),
    "vkvg_close_path": (None, [_P]),
    "vkvg_new_sub_path": (None, [_P]),
    "vkvg_path_extents": (None, [_P, _P, _P, _P, _P]),
    "vkvg_get_current_point": (None, [_P, _P, _P]),
    "vkvg_line_to": (None, [_P, _F, _F]),
    "vkvg_rel_line_to": (None, [_P, _F, _F]),
    "vkvg_move_to": (None, [_P, _F, _F]),
    "vkvg_rel_move_to": (None, [_P, _F, _F]),
    "vkvg_arc": (None, [_P, _F, _F, _F, _F, _F]),
    "vkvg_arc_negative": (None, [_P, _F, _F, _F, _F, _F]),
    "vkvg_curve_to": (None, [_P, _F, _F, _F, _F, _F, _F]),
    "vkvg_rel_curve_to": (None, [_P, _F, _F, _F, _F, _F, _F]),
    "vkvg_quadratic_to": (None, [_P, _F, _F, _F, _F]),
    "vkvg_rel_quadratic_to": (None, [_P, _F, _F, _F, _F]),
    "vkvg_rectangle": (_I, [_P, _F, _F, _F, _F]),
    "vkvg_rounded_rectangle": (_I, [_P, _F, _F, _F, _F, _F]),
    "vkvg_rounded_rectangle2": (None, [_P, _F, _F, _F, _F, _F, _F]),
    "vkvg_ellipse": (None, [_P, _F, _F, _F, _F, _F]),
    "vkvg_elliptic_arc_to": (None, [_P, _F, _F, _B, _B, _F, _F, _F]),
    "vkvg_rel_elliptic_arc_to": (None, [_P, _F, _F, _B, _B, _F, _F, _F]),
    "vkvg_has_current_point": (_B, [_P]),
    "vkvg_stroke": (None, [_P]),
    "vkvg_stroke_preserve": (None, [_P]),
    "vkvg_fill": (None, [_P]),
    "vkvg_fill_preserve": (None, [_P]),
    "vkvg_paint": (None, [_P]),
    "vkvg_clear": (None, [_P]),
    "vkvg_reset_clip": (None, [_P]),
    "vkvg_clip": (None, [_P]),
    "vkvg_clip_preserve": (None, [_P]),
    "vkvg_save": (None, [_P]),
    "vkvg_restore": (None, [_P]),
    "vkvg_set_opacity": (None, [_P, _F]),
    "vkvg_get_opacity": (_F, [_P]),
    "vkvg_set_source_color": (None, [_P, _U]),
    "vkvg_set_source_rgba": (None, [_P, _F, _F, _F, _F]),
    "vkvg_set_source_rgb": (None, [_P, _F, _F, _F]),
    "vkvg_set_source": (None, [_P, _P]),
    "vkvg_get_source": (_P, [_P]),
    "vkvg_pattern_status": (_I, [_P]),
    "vkvg_pattern_reference": (_P, [_P]),
    "vkvg_pattern_get_reference_count": (_U, [_P]),
    "vkvg_pattern_destroy": (None, [_P]),
    "vkvg_pattern_create_linear": (_P, [_F, _F, _F, _F]),
    "vkvg_pattern_edit_linear": (_I, [_P, _F, _F, _F, _F]),
    "vkvg_pattern_create_radial": (_P, [_F, _F, _F, _F, _F, _F]),
    "vkvg_pattern_create_for_surface": (_P, [_P]),
    "vkvg_set_source_surface": (None, [_P, _P, _F, _F]),
    "vkvg_pattern_edit_radial": (_I, [_P, _F, _F, _F, _F, _F, _F]),
    "vkvg_pattern_get_linear_points": (_I, [_P, _P, _P, _P, _P]),
    "vkvg_pattern_add_color_stop": (_I, [_P, _F, _F, _F, _F, _F]),
    "vkvg_pattern_get_color_stop_count": (_I, [_P, _P]),
    "vkvg_pattern_get_color_stop_rgba": (_I, [_P, _U, _P, _P, _P, _P, _P]),
    "vkvg_pattern_set_extend": (None, [_P, _I]),
    "vkvg_pattern_get_extend": (_I, [_P]),
    "vkvg_pattern_set_filter": (None, [_P, _I]),
    "vkvg_pattern_get_filter": (_I, [_P]),
    "vkvg_pattern_get_type": (_I, [_P]),
    "vkvg_pattern_set_matrix": (None, [_P, _P]),
    "vkvg_pattern_get_matrix": (None, [_P, _P]),
    "vkvg_set_line_width": (None, [_P, _F]),
    "vkvg_set_miter_limit": (None, [_P, _F]),
    "vkvg_get_miter_limit": (_F, [_P]),
    "vkvg_set_line_cap": (None, [_P, _I]),
    "vkvg_set_line_join": (None, [_P, _I]),
    "vkvg_set_operator": (None, [_P, _I]),
    "vkvg_set_fill_rule": (None, [_P, _I]),
    "vkvg_set_dash": (None, [_P, _P, _U, _F]),
    "vkvg_get_dash": (None, [_P, _P, _P, _P]),
    "vkvg_get_line_width": (_F, [_P]),
    "vkvg_get_line_cap": (_I, [_P]),
    "vkvg_get_line_join": (_I, [_P]),
    "vkvg_get_operator": (_I, [_P]),
    "vkvg_get_fill_rule": (_I, [_P]),
    "vkvg_get_target": (_P, [_P]),
    "vkvg_translate": (None, [_P, _F, _F]),
    "vkvg_scale": (None, [_P, _F, _F]),
    "vkvg_rotate": (None, [_P, _F]),
    "vkvg_transform": (None, [_P, _P]),
    "vkvg_set_matrix": (None, [_P, _P]),
    "vkvg_get_matrix": (None, [_P, _P]),
    "vkvg_identity_matrix": (None, [_P]),
    # vkvg_gb300.h
    "vkvg_surface_get_device_ptr": (_P, [_P]),
    "vkvg_surface_get_samples": (_U, [_P]),
    "vkvg_gb300_frame_capture": (_P, [_P]),
    "vkvg_gb300_frame_execute": (_I, [_P, _P]),
    "vkvg_gb300_frame_stats": (_I, [_P, _P]),
    "vkvg_gb300_frame_timing": (_I, [_P, _P]),
    "vkvg_gb300_frame_destroy": (None, [_P]),
    "vkvg_gb300_replay_stream": (_I, [_P, _P, _U, _P, C.c_uint64]),
    "vkvg_gb300_debug_capture": (None, [_P, _I]),
    "vkvg_gb300_debug_counts": (_I, [_P, _P]),
    "vkvg_gb300_debug_points": (_I, [_P, _P, _P]),
    "vkvg_gb300_debug_subpaths": (_I, [_P, _P, _P, _P]),
    "vkvg_gb300_debug_draw": (_I, [_P, _U, _P]),
    "vkvg_gb300_debug_stroke": (_I, [_P, _U, _P, _P]),
    "vkvg_gb300_debug_coverage": (_I, [_P, _U, _P]),
    "vkvg_gb300_debug_set_raster_form": (None, [_I]),
    "vkvg_gb300_debug_raster_form": (_I, [_P]),
    "vkvg_gb300_debug_inject": (None, [_I, _U]),
    "vkvg_gb300_surface_read_samples": (_I, [_P, _P]),
    "vkvg_gb300_surface_read_premult": (_I, [_P, _P]),
    "vkvg_gb300_pmath_eval": (_I, [_I, _P, _P, _P, C.c_uint64, _I]),
    "vkvg_gb300_kernel_launches": (C.c_uint64, []),
    "vkvg_gb300_exclusive_scan_noalloc": (_I, [_P, _P, C.c_uint32, _P]),
    "vkvg_gb300_batch_create": (_P, [_P, _P, _U]),
    "vkvg_gb300_batch_execute": (_I, [_P]),
    "vkvg_gb300_batch_timing": (_I, [_P, _P]),
    "vkvg_gb300_batch_destroy": (None, [_P]),
    # include/vkvg-svg.h
    "vkvg_svg_load": (_P, [C.c_char_p]),
    "vkvg_svg_load_fragment": (_P, [C.c_char_p]),
    "vkvg_svg_destroy": (None, [_P]),
    "vkvg_svg_get_dimensions": (None, [_P, _P, _P]),
    "vkvg_svg_render": (None, [_P, _P, C.c_char_p]),
    "vkvg_surface_create_from_svg": (_P, [_P, _U, _U, C.c_char_p]),
    "vkvg_surface_create_from_svg_fragment": (_P, [_P, _U, _U, C.c_char_p]),
    "vkvg_gb300_svg_shape_count": (_U, [_P]),
    "vkvg_gb300_svg_shape": (_I, [_P, _U, _P, _P, _P]),
    "vkvg_gb300_svg_path": (_I, [_P, _U, _U, _P, _U, _P, _P]),
    "vkvg_gb300_analytic_create": (_P, [_U, _U, _P, _U, _P, _P, _U, _P, _U, _P]),
    "vkvg_gb300_analytic_create_tiled": (_P, [_U, _U, _U, _P, _U, _P, _P, _U, _P, _U, _P]),
    "vkvg_gb300_analytic_destroy": (None, [_P]),
    "vkvg_gb300_analytic_status": (_I, [_P]),
    "vkvg_gb300_analytic_control_point_count": (_U, [_P]),
    "vkvg_gb300_analytic_layer_count": (_U, [_P]),
    "vkvg_gb300_analytic_set_stream": (_I, [_P, _P]),
    "vkvg_gb300_analytic_forward": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "vkvg_gb300_analytic_backward": (_I, [_P, _P, _P, _P, _P]),
    "vkvg_gb300_analytic_adam": (_I, [_P, _P, _P, _P, _P, _U, _F, _F, _F, _F, _U, _F, _F]),
    "vkvg_gb300_analytic_sync": (_I, [_P]),
    "vkvg_gb300_analytic_points": (_U, [_P, _P, _U, _P]),
    "vkvg_gb300_analytic_point_grads": (_U, [_P, _P, _U]),
    "vkvg_gb300_analytic_set_timing": (_I, [_P, _I]),
    "vkvg_gb300_analytic_timing": (_I, [_P, _P]),
}


class Matrix(C.Structure):
    _fields_ = [("xx", _F), ("yx", _F), ("xy", _F), ("yy", _F), ("x0", _F), ("y0", _F)]


class DeviceCreateInfo(C.Structure):
    _fields_ = [("samples", C.c_uint32), ("deferredResolve", C.c_bool), ("inst", _P), ("phy", _P),
                ("vkdev", _P), ("qFamIdx", C.c_uint32), ("qIndex", C.c_uint32), ("threadAware", C.c_bool)]


def lib():
    """Load libvkvg_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libvkvg_gb300.so is missing (%s); run __graft_entry__.build() or "
                               "python vkvg_gb300/build.py" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class VkvgError(RuntimeError):
    pass


class Device:
    def __init__(self, samples=4, thread_aware=False):
        L = lib()
        info = DeviceCreateInfo(samples=samples, threadAware=thread_aware)
        self.h = L.vkvg_device_create(C.byref(info))
        st = L.vkvg_device_status(self.h)
        if st:
            raise VkvgError("vkvg_device_create failed: %s" % L.vkvg_status_to_string(st).decode())

    def destroy(self):
        if self.h:
            lib().vkvg_device_destroy(self.h)
            self.h = None


class Surface:
    def __init__(self, dev, width, height):
        L = lib()
        self.dev = dev
        self.h = L.vkvg_surface_create(dev.h, width, height)
        st = L.vkvg_surface_status(self.h)
        if st:
            raise VkvgError("vkvg_surface_create failed: %s" % L.vkvg_status_to_string(st).decode())
        self.width, self.height = width, height
        self.samples = L.vkvg_surface_get_samples(self.h)

    def image(self):
        """vkvg_surface_write_to_memory: resolved, unpremultiplied RGBA8."""
        out = np.zeros((self.height, self.width, 4), np.uint8)
        st = lib().vkvg_surface_write_to_memory(self.h, _ptr(out))
        if st:
            raise VkvgError("write_to_memory: %d" % st)
        return out

    def premult(self):
        out = np.zeros((self.height, self.width, 4), np.uint8)
        lib().vkvg_gb300_surface_read_premult(self.h, _ptr(out))
        return out

    def samples_rgba(self):
        out = np.zeros((self.height, self.width, self.samples, 4), np.uint8)
        lib().vkvg_gb300_surface_read_samples(self.h, _ptr(out))
        return out

    def write_png(self, path):
        return lib().vkvg_surface_write_to_png(self.h, path.encode())

    def context(self):
        return Context(self)

    def destroy(self):
        if self.h:
            lib().vkvg_surface_destroy(self.h)
            self.h = None


class Context:
    """vkvg context; unknown attributes map to vkvg_<name>(ctx, ...)."""

    def __init__(self, surf):
        self.L = lib()
        self.surf = surf
        self.h = self.L.vkvg_create(surf.h)
        st = self.L.vkvg_status(self.h)
        if st:
            raise VkvgError("vkvg_create failed: %d" % st)

    def __getattr__(self, name):
        fn = getattr(self.L, "vkvg_" + name)
        return lambda *a: fn(self.h, *a)

    def set_dash(self, dashes, offset):
        arr = np.asarray(dashes, dtype=np.float32)
        self.L.vkvg_set_dash(self.h, _ptr(arr) if len(arr) else None, len(arr), offset)

    def set_matrix(self, m):
        mm = Matrix(*m)
        self.L.vkvg_set_matrix(self.h, C.byref(mm))

    def set_source_linear(self, x0, y0, x1, y1, stops, pmat=None):
        """a linear gradient pattern as the source (created, used, released)"""
        p = self.L.vkvg_pattern_create_linear(x0, y0, x1, y1)
        for st in stops:
            self.L.vkvg_pattern_add_color_stop(p, *st)
        if pmat is not None:
            mm = Matrix(*pmat)
            self.L.vkvg_pattern_set_matrix(p, C.byref(mm))
        self.L.vkvg_set_source(self.h, p)
        self.L.vkvg_pattern_destroy(p)

    def set_source_surface(self, surf, x, y):
        self.L.vkvg_set_source_surface(self.h, surf.h, x, y)

    def set_source_surface_pattern(self, surf, extend, filt, pmat=None):
        """a surface pattern with sampler settings as the source (created,
        used, released)"""
        p = self.L.vkvg_pattern_create_for_surface(surf.h)
        self.L.vkvg_pattern_set_extend(p, extend)
        self.L.vkvg_pattern_set_filter(p, filt)
        if pmat is not None:
            mm = Matrix(*pmat)
            self.L.vkvg_pattern_set_matrix(p, C.byref(mm))
        self.L.vkvg_set_source(self.h, p)
        self.L.vkvg_pattern_destroy(p)

    def set_source_radial(self, cx0, cy0, r0, cx1, cy1, r1, stops, pmat=None):
        """a radial gradient pattern as the source (created, used, released)"""
        p = self.L.vkvg_pattern_create_radial(cx0, cy0, r0, cx1, cy1, r1)
        for st in stops:
            self.L.vkvg_pattern_add_color_stop(p, *st)
        if pmat is not None:
            mm = Matrix(*pmat)
            self.L.vkvg_pattern_set_matrix(p, C.byref(mm))
        self.L.vkvg_set_source(self.h, p)
        self.L.vkvg_pattern_destroy(p)

    def current_point(self):
        x, y = C.c_float(), C.c_float()
        self.L.vkvg_get_current_point(self.h, C.byref(x), C.byref(y))
        return x.value, y.value

    def debug_capture(self, on=True):
        self.L.vkvg_gb300_debug_capture(self.h, 1 if on else 0)

    def debug_counts(self):
        out = np.zeros(8, np.uint32)
        self.L.vkvg_gb300_debug_counts(self.h, _ptr(out))
        return out

    def debug_points(self):
        n = int(self.debug_counts()[1])
        xy = np.zeros((max(n, 1), 2), np.float32)
        fl = np.zeros(max(n, 1), np.uint8)
        self.L.vkvg_gb300_debug_points(self.h, _ptr(xy), _ptr(fl))
        return xy[:n], fl[:n]

    def debug_subpaths(self):
        n = int(self.debug_counts()[0])
        a = np.zeros(max(n, 1), np.uint32)
        b = np.zeros(max(n, 1), np.uint32)
        c = np.zeros(max(n, 1), np.uint32)
        self.L.vkvg_gb300_debug_subpaths(self.h, _ptr(a), _ptr(b), _ptr(c))
        return a[:n], b[:n], c[:n]

    def debug_draw(self, i):
        info = np.zeros(8, np.uint32)
        st = self.L.vkvg_gb300_debug_draw(self.h, i, _ptr(info))
        if st:
            raise VkvgError("debug_draw %d: %d" % (i, st))
        return info

    def debug_stroke(self, i):
        info = self.debug_draw(i)
        nv, ni = int(info[3]), int(info[4])
        v = np.zeros((max(nv, 1), 2), np.float32)
        ix = np.zeros(max(ni, 1), np.uint32)
        st = self.L.vkvg_gb300_debug_stroke(self.h, i, _ptr(v), _ptr(ix))
        if st:
            raise VkvgError("debug_stroke %d: %d" % (i, st))
        return v[:nv], ix[:ni]

    def raster_form(self):
        """the raster form the last flush ran (0 1024-pixel register tile,
        1 256-pixel, 2 128-pixel, 3 row form in half bands, 4 in whole bands)"""
        return int(self.L.vkvg_gb300_debug_raster_form(self.h))

    def debug_coverage(self, i):
        s = self.surf
        out = np.zeros((s.height, s.width, s.samples), np.int32)
        st = self.L.vkvg_gb300_debug_coverage(self.h, i, _ptr(out))
        if st:
            raise VkvgError("debug_coverage %d: %d" % (i, st))
        return out

    def destroy(self):
        if self.h:
            self.L.vkvg_destroy(self.h)
            self.h = None


def kernel_launches():
    return int(lib().vkvg_gb300_kernel_launches())


SCAN_NOALLOC_MAX = 1 << 26


def exclusive_scan_noalloc(counts_ptr, n, offsets_ptr, stream=0):
    """Device exclusive scan of n uint32 counts into n + 1 offsets without
    allocating (device pointers as ints); returns the vkvg status code."""
    return int(lib().vkvg_gb300_exclusive_scan_noalloc(C.c_void_p(stream), C.c_void_p(counts_ptr), n,
                                                        C.c_void_p(offsets_ptr)))


def pmath(fn, a, b=None, device=False):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(a if b is None else b, np.float32)
    out = np.empty_like(a)
    st = lib().vkvg_gb300_pmath_eval(fn, _ptr(a), _ptr(b), _ptr(out), a.size, 1 if device else 0)
    if st:
        raise VkvgError("pmath_eval: %d" % st)
    return out


class Svg:
    """A parsed SVG document (include/vkvg-svg.h): vkvg_svg_load_fragment of
    `text` (bytes), rendered with render(ctx, id)."""

    def __init__(self, text):
        self.L = lib()
        self.h = self.L.vkvg_svg_load_fragment(text)
        if not self.h:
            raise VkvgError("vkvg_svg_load_fragment failed")

    def dimensions(self):
        w, h = C.c_uint32(), C.c_uint32()
        self.L.vkvg_svg_get_dimensions(self.h, C.byref(w), C.byref(h))
        return w.value, h.value

    def render(self, ctx, sub_id=None):
        self.L.vkvg_svg_render(self.h, ctx.h, sub_id)

    def shapes(self):
        """what vkvg's SVG walk reads, per shape: id, fill / stroke paint type
        and colour, visibility, opacity, stroke width, bounds, and the paths
        as (float32 points [n, 2], closed)"""
        out = []
        for i in range(self.L.vkvg_gb300_svg_shape_count(self.h)):
            idb = C.create_string_buffer(64)
            u = np.zeros(6, np.uint32)
            f = np.zeros(6, np.float32)
            self.L.vkvg_gb300_svg_shape(self.h, i, idb, _ptr(u), _ptr(f))
            paths = []
            for p in range(int(u[5])):
                n, closed = C.c_uint32(), C.c_uint32()
                self.L.vkvg_gb300_svg_path(self.h, i, p, None, 0, C.byref(n), C.byref(closed))
                pts = np.zeros((max(n.value, 1), 2), np.float32)
                self.L.vkvg_gb300_svg_path(self.h, i, p, _ptr(pts), n.value, C.byref(n), C.byref(closed))
                paths.append((pts[:n.value], bool(closed.value)))
            out.append({"id": idb.value, "fill_type": int(u[0]), "fill_color": int(u[1]), "stroke_type": int(u[2]),
                        "stroke_color": int(u[3]), "visible": bool(u[4]), "opacity": f[0], "stroke_width": f[1],
                        "bounds": f[2:6].copy(), "paths": paths})
        return out

    def destroy(self):
        if self.h:
            self.L.vkvg_svg_destroy(self.h)
            self.h = None


class Analytic:
    """Differentiable analytic-coverage scene (vkvg_gb300_analytic_* of
    include/vkvg_gb300.h) for a scene description of
    vkvg_gb300.scenes.analytic_scene.  Parameters and results are CUDA
    tensors (float32, contiguous); the calls are queued on the tensors'
    current stream."""

    def __init__(self, scene, tile=0):
        """tile > 0: the tiled evaluation (vkvg_gb300_analytic_create_tiled)"""
        import torch

        self.L = lib()
        self.torch = torch
        s = {k: np.ascontiguousarray(v) for k, v in scene.items() if isinstance(v, np.ndarray)}
        self._keep = s
        self.W, self.H = int(scene["width"]), int(scene["height"])
        self.npaths = len(s["path_ncontours"])
        args = (_ptr(s["background"].astype(np.float32)), self.npaths, _ptr(s["path_ncontours"]),
                _ptr(s["path_flags"]), len(s["contour_nseg"]), _ptr(s["contour_nseg"]), len(s["seg_kind"]),
                _ptr(s["seg_kind"]))
        if tile:
            self.h = self.L.vkvg_gb300_analytic_create_tiled(self.W, self.H, tile, *args)
        else:
            self.h = self.L.vkvg_gb300_analytic_create(self.W, self.H, *args)
        if not self.h:
            raise VkvgError("vkvg_gb300_analytic_create failed")
        self.nctrl = self.L.vkvg_gb300_analytic_control_point_count(self.h)
        self.nlayers = self.L.vkvg_gb300_analytic_layer_count(self.h)
        self.L.vkvg_gb300_analytic_set_stream(self.h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        self.canvas = torch.empty((self.H, self.W, 4), dtype=torch.float32, device="cuda")
        self.loss = torch.zeros(1, dtype=torch.float32, device="cuda")

    @staticmethod
    def _p(t):
        return C.c_void_p(t.data_ptr()) if t is not None else None

    def _shape(self, name, t, n):
        t_ = self.torch
        if t.dtype != t_.float32 or not t.is_contiguous() or t.numel() != n or t.device.type != "cuda":
            raise VkvgError("%s: want %d contiguous float32 values on the GPU, got %s %s of %d on %s"
                            % (name, n, t.dtype, "contiguous" if t.is_contiguous() else "strided", t.numel(),
                               t.device))

    def _check(self, st, what):
        if st:
            raise VkvgError("%s: status %d" % (what, st))

    def forward(self, ctrl, colors, widths, target=None):
        """renders into self.canvas (and the loss into self.loss when a target
        is given); returns (canvas, loss or None).  The tensors must be this
        scene's: float32, contiguous, on the GPU, ctrl of its control points,
        colors and widths of its paths, target of its canvas (the kernels
        index them by the scene's structure)."""
        self._shape("ctrl", ctrl, 2 * self.nctrl)
        self._shape("colors", colors, 4 * self.npaths)
        self._shape("widths", widths, self.npaths)
        if target is not None:
            self._shape("target", target, 4 * self.W * self.H)
        p = self._p
        st = self.L.vkvg_gb300_analytic_forward(self.h, p(ctrl), p(colors), p(widths), p(target), p(self.canvas),
                                                p(self.loss) if target is not None else None)
        self._check(st, "analytic_forward")
        self._keep_fwd = (ctrl, colors, widths, target)
        return self.canvas, (self.loss if target is not None else None)

    def backward(self, d_canvas=None, grads=None):
        """gradients of the last forward's loss (d_canvas None) or of
        sum(d_canvas * canvas): (d_ctrl, d_colors, d_widths)"""
        t = self.torch
        if grads is None:
            grads = (t.empty((self.nctrl, 2), dtype=t.float32, device="cuda"),
                     t.empty((self.npaths, 4), dtype=t.float32, device="cuda"),
                     t.empty(self.npaths, dtype=t.float32, device="cuda"))
        if d_canvas is not None:
            self._shape("d_canvas", d_canvas, 4 * self.W * self.H)
        for name, g, n in zip(("d_ctrl", "d_colors", "d_widths"), grads, (2 * self.nctrl, 4 * self.npaths, self.npaths)):
            self._shape(name, g, n)
        p = self._p
        st = self.L.vkvg_gb300_analytic_backward(self.h, p(d_canvas), p(grads[0]), p(grads[1]), p(grads[2]))
        self._check(st, "analytic_backward")
        return grads

    def adam(self, param, grad, m, v, step, lr, lo, hi, beta1=0.9, beta2=0.999, eps=1e-8):
        st = self.L.vkvg_gb300_analytic_adam(self.h, self._p(param), self._p(grad), self._p(m), self._p(v),
                                             param.numel(), lr, beta1, beta2, eps, step, lo, hi)
        self._check(st, "analytic_adam")

    def sync(self):
        return int(self.L.vkvg_gb300_analytic_sync(self.h))

    def points(self):
        n = self.L.vkvg_gb300_analytic_points(self.h, None, 0, None)
        pts = np.zeros((max(n, 1), 2), np.float32)
        off = np.zeros(len(self._keep["seg_kind"]) + 1, np.uint32)
        self.L.vkvg_gb300_analytic_points(self.h, _ptr(pts), n, _ptr(off))
        return pts[:n], off

    def set_timing(self, on=True):
        self._check(self.L.vkvg_gb300_analytic_set_timing(self.h, 1 if on else 0), "analytic_set_timing")

    def timing(self):
        """ms of the last forward's flattening, coverage, compositing and the
        last backward's compositing, coverage and flattening adjoints"""
        t = np.zeros(6, np.float32)
        self._check(self.L.vkvg_gb300_analytic_timing(self.h, _ptr(t)), "analytic_timing")
        return t

    def point_grads(self):
        """dL/dpoint of the last backward, float32 [points, 2]"""
        n = self.L.vkvg_gb300_analytic_point_grads(self.h, None, 0)
        g = np.zeros((max(n, 1), 2), np.float32)
        self.L.vkvg_gb300_analytic_point_grads(self.h, _ptr(g), n)
        return g[:n]

    def destroy(self):
        if self.h:
            self.L.vkvg_gb300_analytic_destroy(self.h)
            self.h = None
