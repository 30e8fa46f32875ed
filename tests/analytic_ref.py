"""ctypes binding of the FP64 reference of the analytic-coverage mode
(oracle/vko_analytic.c) for the tests and the bench's CPU-baseline leg.  Test
infrastructure: the product package never imports this module."""
import ctypes as C

import numpy as np

import oracle_bind

_P, _U, _D = C.c_void_p, C.c_uint32, C.c_double
_SIGS = {
    "vko_an_create": (_P, [_U, _U, _P, _U, _P, _P, _U, _P, _U, _P]),
    "vko_an_destroy": (None, [_P]),
    "vko_an_nctrl": (_U, [_P]),
    "vko_an_nlayers": (_U, [_P]),
    "vko_an_flatten": (_U, [_P, _P, _P, _P, _U, _P]),
    "vko_an_forward": (_D, [_P, _P, _P, _P, _P, _P, _P]),
    "vko_an_backward": (_D, [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "vko_an_fd": (None, [_P, _P, _P, _P, _P, _U, _P, _P, _D, _D, C.c_int, C.c_int, _P, _P, _P]),
}
_lib = None


def lib():
    global _lib
    if _lib is None:
        L = oracle_bind.lib()
        for k, (r, a) in _SIGS.items():
            f = getattr(L, k)
            f.restype, f.argtypes = r, a
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _f64(a, n=None):
    """a as contiguous float64; n: the number of values it must hold (the C
    reference indexes it by the scene's structure)"""
    a = np.ascontiguousarray(a, np.float64)
    if n is not None and a.size != n:
        raise ValueError("want %d values, got %d" % (n, a.size))
    return a


class Reference:
    """The FP64 reference for one scene description (vkvg_gb300.scenes.analytic_scene)"""

    def __init__(self, scene):
        L = lib()
        self.s = {k: np.ascontiguousarray(v) for k, v in scene.items() if isinstance(v, np.ndarray)}
        s = self.s
        self.W, self.H = int(scene["width"]), int(scene["height"])
        self.npaths = len(s["path_ncontours"])
        self.h = L.vko_an_create(self.W, self.H, _p(s["background"].astype(np.float32)), self.npaths,
                                 _p(s["path_ncontours"]), _p(s["path_flags"]), len(s["contour_nseg"]),
                                 _p(s["contour_nseg"]), len(s["seg_kind"]), _p(s["seg_kind"]))
        if not self.h:
            raise ValueError("invalid analytic scene")
        self.nctrl = L.vko_an_nctrl(self.h)
        self.nlayers = L.vko_an_nlayers(self.h)

    def close(self):
        if self.h:
            lib().vko_an_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _ctrl(self, ctrl):
        return _f64(ctrl, 2 * self.nctrl)

    def flatten(self, ctrl):
        ctrl = self._ctrl(ctrl)
        seg = np.zeros(len(self.s["seg_kind"]) + 1, np.uint32)
        n = lib().vko_an_flatten(self.h, _p(ctrl), None, None, 0, _p(seg))
        f32 = np.zeros((max(n, 1), 2), np.float32)
        f64 = np.zeros((max(n, 1), 2), np.float64)
        lib().vko_an_flatten(self.h, _p(ctrl), _p(f32), _p(f64), n, None)
        return f32[:n], f64[:n], seg

    def forward(self, ctrl, colors, widths, target=None, area=False):
        canvas = np.zeros((self.H, self.W, 4), np.float64)
        A = np.zeros((self.nlayers, self.H, self.W), np.float64) if area else None
        t = _f64(target, 4 * self.W * self.H) if target is not None else None
        loss = lib().vko_an_forward(self.h, _p(self._ctrl(ctrl)), _p(_f64(colors, 4 * self.npaths)),
                                    _p(_f64(widths, self.npaths)), _p(t),
                                    _p(canvas), _p(A))
        return (canvas, loss, A) if area else (canvas, loss)

    def backward(self, ctrl, colors, widths, target=None, d_canvas=None, points=False):
        """(loss, d_ctrl, d_colors, d_widths[, d_points])"""
        d_ctrl = np.zeros((self.nctrl, 2), np.float64)
        d_col = np.zeros((self.npaths, 4), np.float64)
        d_w = np.zeros(self.npaths, np.float64)
        d_pts = np.zeros((max(len(self.flatten(ctrl)[0]), 1), 2), np.float64) if points else None
        t = _f64(target, 4 * self.W * self.H) if target is not None else None
        g = _f64(d_canvas, 4 * self.W * self.H) if d_canvas is not None else None
        loss = lib().vko_an_backward(self.h, _p(self._ctrl(ctrl)), _p(_f64(colors, 4 * self.npaths)),
                                     _p(_f64(widths, self.npaths)), _p(t), _p(g),
                                     _p(d_ctrl), _p(d_col), _p(d_w), _p(d_pts))
        return (loss, d_ctrl, d_col, d_w, d_pts) if points else (loss, d_ctrl, d_col, d_w)

    def fd(self, ctrl, colors, widths, target, group, index, h=1e-3, h2=0.0, full=False, threads=None):
        """central differences of the MSE loss at step h (and at h2 when h2 >
        0); group 0 ctrl coordinate (2*cp + axis), 1 colour (4*path +
        channel), 2 width (path).  Returns (fd, valid) or (fd, fd2, valid);
        valid is False where the flattening changes within the step."""
        import os

        group = np.ascontiguousarray(group, np.uint32)
        index = np.ascontiguousarray(index, np.uint32)
        out = np.zeros(len(group), np.float64)
        out2 = np.zeros(len(group), np.float64)
        ok = np.zeros(len(group), np.int32)
        threads = threads or min(16, os.cpu_count() or 1)
        lib().vko_an_fd(self.h, _p(self._ctrl(ctrl)), _p(_f64(colors, 4 * self.npaths)), _p(_f64(widths, self.npaths)),
                        _p(_f64(target, 4 * self.W * self.H)), len(group),
                        _p(group), _p(index), h, h2, int(full), threads, _p(out), _p(out2), _p(ok))
        return (out, ok.astype(bool)) if h2 <= 0 else (out, out2, ok.astype(bool))
