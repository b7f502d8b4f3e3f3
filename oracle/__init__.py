"""TEST INFRASTRUCTURE ONLY — ctypes wrapper of the CPU oracle (footile_oracle.cpp).

The oracle is a sequential C++ restatement of footile's fill/stroke path.  Only
tests/, __graft_entry__.smoke() and bench.py (cpu_baseline leg and the
`--impl reference` arm) use it, as the test oracle and CPU baseline.  The shipped
library (footile_gb300) never imports it.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

from footile_gb300 import _abi

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libfootile_oracle.so")
_lock = threading.Lock()
_lib = None


def build():
    """Compile the oracle (g++, a few seconds)."""
    subprocess.check_call(["make", "-s", "-C", _HERE])


class Params(ctypes.Structure):
    _fields_ = [("tolerance", ctypes.c_float), ("transform", ctypes.c_float * 6),
                ("join", ctypes.c_int32), ("miter_limit", ctypes.c_float), ("fig_cap", ctypes.c_uint32)]


def make_params(tolerance=0.3, transform=_abi.IDENTITY, join=_abi.JOIN_MITER, miter_limit=4.0, fig_cap=0):
    """`fig_cap` above 65,535: fills keep that many vertices per figure (u32 vertex ids),
    the un-capped extension; 0 is footile's 65,535-vertex Fig."""
    p = Params()
    p.tolerance = tolerance
    for i in range(6):
        p.transform[i] = transform[i]
    p.join = join
    p.miter_limit = miter_limit
    p.fig_cap = fig_cap
    return p


def lib():
    global _lib
    with _lock:
        if _lib is None:
            src = os.path.join(_HERE, "footile_oracle.cpp")
            if not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
                build()
            L = ctypes.CDLL(_SO)
            P = ctypes.c_void_p
            i32, u32 = ctypes.c_int32, ctypes.c_uint32
            L.orc_fill.argtypes = [i32, P, u32, i32, P, P, u32, u32, u32, ctypes.POINTER(Params),
                                   ctypes.POINTER(ctypes.c_float)]
            L.orc_fill.restype = ctypes.c_int
            L.orc_stroke.argtypes = [P, u32, i32, P, P, u32, u32, u32, ctypes.POINTER(Params),
                                     ctypes.POINTER(ctypes.c_float)]
            L.orc_stroke.restype = ctypes.c_int
            L.orc_stroke_outline.argtypes = [P, u32, ctypes.POINTER(Params), ctypes.c_float, P, u32]
            L.orc_stroke_outline.restype = u32
            L.orc_stroke_points.argtypes = [P, u32, ctypes.POINTER(Params), ctypes.c_float, P, P,
                                            ctypes.POINTER(u32), P, ctypes.POINTER(u32), u32]
            L.orc_stroke_points.restype = u32
            L.orc_join_decisions.argtypes = [P, u32, ctypes.POINTER(Params), ctypes.c_float, i32, P, P, u32]
            L.orc_join_decisions.restype = u32
            L.orc_fig_points.argtypes = [P, u32, ctypes.POINTER(Params), P, u32]
            L.orc_fig_points.restype = u32
            L.orc_accumulate.argtypes = [i32, P, P, u32]
            L.orc_accumulate.restype = None
            L.orc_fx_from_f32.argtypes = [ctypes.c_float]
            L.orc_fx_from_f32.restype = i32
            L.orc_fx_from_int.argtypes = [i32]
            L.orc_fx_from_int.restype = i32
            L.orc_fx_to_f32.argtypes = [i32]
            L.orc_fx_to_f32.restype = ctypes.c_float
            L.orc_fx_to_int.argtypes = [i32]
            L.orc_fx_to_int.restype = i32
            L.orc_fx_op.argtypes = [i32, i32, i32]
            L.orc_fx_op.restype = i32
            L.orc_widdershins.argtypes = [i32, i32, i32, i32]
            L.orc_widdershins.restype = i32
            L.orc_atan2f.argtypes = [ctypes.c_float, ctypes.c_float]
            L.orc_atan2f.restype = ctypes.c_float
            L.orc_sinf.argtypes = [ctypes.c_float]
            L.orc_sinf.restype = ctypes.c_float
            L.orc_fill_batch.argtypes = [i32, i32, P, P, u32, i32, P, ctypes.POINTER(Params), P, i32]
            L.orc_fill_batch.restype = ctypes.c_int
            L.orc_composite.argtypes = [i32, i32, P, P, u32, i32, P, u32, u32, u32, ctypes.POINTER(Params),
                                        ctypes.POINTER(ctypes.c_float), P]
            L.orc_composite.restype = ctypes.c_int
            D = ctypes.POINTER(ctypes.c_double)
            L.orc_adj_forward.argtypes = [i32, P, u32, P, u32, u32, ctypes.c_float, P, P, P]
            L.orc_adj_forward.restype = ctypes.c_int
            L.orc_adj_backward.argtypes = [i32, P, u32, P, u32, u32, ctypes.c_float, P, P, P, P]
            L.orc_adj_backward.restype = ctypes.c_int
            d = ctypes.c_double
            L.orc_adj_stroke_forward.argtypes = [P, u32, P, d, u32, u32, ctypes.c_float, P, i32, ctypes.c_float, P, P]
            L.orc_adj_stroke_forward.restype = ctypes.c_int
            L.orc_adj_stroke_backward.argtypes = [P, u32, P, d, u32, u32, ctypes.c_float, P, i32, ctypes.c_float, P, P,
                                                  P, ctypes.POINTER(d)]
            L.orc_adj_stroke_backward.restype = ctypes.c_int
            L.orc_adj_stroke_outline.argtypes = [P, u32, ctypes.c_float, P, i32, ctypes.c_float, ctypes.c_float, P, u32]
            L.orc_adj_stroke_outline.restype = u32
            del D
            _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _clr(clr):
    return np.ascontiguousarray(np.asarray(clr if clr is not None else (0, 0, 0, 0), dtype=np.uint8))


def fill(rule, ops, raster, fmt, clr=None, s_width=1.0, **params):
    """Plotter::fill on `raster` (modified in place).  Returns (status, s_width)."""
    ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
    assert raster.flags.c_contiguous
    h = raster.shape[0]
    w = raster.shape[1]
    stride = raster.strides[0]
    c = _clr(clr)
    sw = ctypes.c_float(s_width)
    st = lib().orc_fill(rule, _ptr(ops), len(ops), fmt, _ptr(c), _ptr(raster), w, h, stride,
                        ctypes.byref(make_params(**params)), ctypes.byref(sw))
    return st, sw.value


def stroke(ops, raster, fmt, clr=None, s_width=1.0, **params):
    """Plotter::stroke on `raster` (modified in place).  Returns (status, s_width)."""
    ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
    h = raster.shape[0]
    w = raster.shape[1]
    stride = raster.strides[0]
    c = _clr(clr)
    sw = ctypes.c_float(s_width)
    st = lib().orc_stroke(_ptr(ops), len(ops), fmt, _ptr(c), _ptr(raster), w, h, stride,
                          ctypes.byref(make_params(**params)), ctypes.byref(sw))
    return st, sw.value


def stroke_outline(ops, s_width=1.0, **params):
    ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
    cap = 1 << 16
    while True:
        out = np.zeros(cap, dtype=_abi.OP_DTYPE)
        n = lib().orc_stroke_outline(_ptr(ops), len(ops), ctypes.byref(make_params(**params)), s_width,
                                     _ptr(out), cap)
        if n <= cap:
            return out[:n]
        cap = n


def stroke_points(ops, s_width=1.0, **params):
    """The stroker's input and result for `ops` (stroker.rs:204-236): the events the
    plotter hands it, an (n, 4) f32 array of (x, y, width, 0) per add_point and
    (0, 0, 0, 1 + joined) per close; the kept stroke points, (m, 3) f32 (x, y, width);
    and the sub-strokes, (k, 4) int32 (start, points, joined, done)."""
    ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
    cap = 1 << 16
    while True:
        ev = np.zeros((cap, 4), np.float32)
        pts = np.zeros((cap, 3), np.float32)
        subs = np.zeros((cap, 4), np.int32)
        n_pts, n_subs = ctypes.c_uint32(0), ctypes.c_uint32(0)
        n = lib().orc_stroke_points(_ptr(ops), len(ops), ctypes.byref(make_params(**params)), s_width, _ptr(ev),
                                    _ptr(pts), ctypes.byref(n_pts), _ptr(subs), ctypes.byref(n_subs), cap)
        if max(n, n_pts.value, n_subs.value) <= cap:
            return ev[:n].copy(), pts[:n_pts.value].copy(), subs[:n_subs.value].copy()
        cap = max(n, n_pts.value, n_subs.value)


def join_decisions(ops, s_width=1.0, libm=False, with_uv=False, **params):
    """The stroke outline's join decisions in order (0 bevel, 1 miter, 2 round arc), taken
    by ft_fmath.h as a correctly rounded f32 libm takes them (libm=False, the CUDA path's
    decisions) or with the C library's atan2f / sinf (libm=True).  with_uv: also the
    joins' vectors u = a1 - a0, v = b0 - b1 as an (n, 4) f32 array."""
    ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
    cap = 1 << 16
    while True:
        out = np.zeros(cap, dtype=np.int8)
        uv = np.zeros((cap, 4), dtype=np.float32) if with_uv else None
        n = lib().orc_join_decisions(_ptr(ops), len(ops), ctypes.byref(make_params(**params)), s_width,
                                     int(bool(libm)), _ptr(out), _ptr(uv) if with_uv else None, cap)
        if n <= cap:
            return (out[:n], uv[:n]) if with_uv else out[:n]
        cap = n


def fig_points(ops, **params):
    """The Fixed (16.16) vertices footile's Fig holds after the path walk."""
    ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
    xy = np.zeros((_abi.MAX_POINTS, 2), dtype=np.int32)
    n = lib().orc_fig_points(_ptr(ops), len(ops), ctypes.byref(make_params(**params)), _ptr(xy),
                             _abi.MAX_POINTS)
    return xy[:n].copy()


def accumulate(rule, src):
    """imgbuf accumulate_non_zero / accumulate_even_odd: returns (dst, src_after)."""
    s = np.ascontiguousarray(np.array(src, dtype=np.int16))
    d = np.zeros(len(s), dtype=np.uint8)
    lib().orc_accumulate(rule, _ptr(s), _ptr(d), len(s))
    return d, s


def fill_batch(stroke, rule, ops, paths, fmt, rasters, n_threads=1, **params):
    ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
    paths = np.ascontiguousarray(paths, dtype=_abi.PATH_DTYPE)
    status = np.zeros(len(paths), dtype=np.int32)
    lib().orc_fill_batch(stroke, rule, _ptr(ops), _ptr(paths), len(paths), fmt, _ptr(rasters),
                         ctypes.byref(make_params(**params)), _ptr(status), n_threads)
    return status


# Fixed (16.16) arithmetic of fixed.rs, for the known-answer tests
FX_ADD, FX_SUB, FX_MUL, FX_DIV, FX_SHL, FX_SHR, FX_ABS, FX_FLOOR, FX_CEIL, FX_ROUND, FX_TRUNC, \
    FX_FRACT, FX_AVG = range(13)


def fx(v):
    """Fixed::from(f32) for floats, Fixed::from(i32) for ints."""
    if isinstance(v, (int, np.integer)):
        return lib().orc_fx_from_int(int(v))
    return lib().orc_fx_from_f32(float(v))


def fx_op(op, a, b=0):
    return lib().orc_fx_op(op, a, b)


def fx_to_f32(v):
    return lib().orc_fx_to_f32(v)


def fx_to_int(v):
    return lib().orc_fx_to_int(v)


def widdershins(a, b):
    return bool(lib().orc_widdershins(a[0], a[1], b[0], b[1]))


def atan2f(y, x):
    return lib().orc_atan2f(y, x)


def sinf(x):
    return lib().orc_sinf(x)


def composite(stroke, rule, ops, paths, fmt, raster, s_width=1.0, **params):
    """Plotter calls one after another on one raster; returns (status array, s_width)."""
    ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
    paths = np.ascontiguousarray(paths, dtype=_abi.PATH_DTYPE)
    status = np.zeros(len(paths), dtype=np.int32)
    sw = ctypes.c_float(s_width)
    h, w = raster.shape[0], raster.shape[1]
    lib().orc_composite(stroke, rule, _ptr(ops), _ptr(paths), len(paths), fmt, _ptr(raster), w, h,
                        raster.strides[0], ctypes.byref(make_params(**params)), ctypes.byref(sw), _ptr(status))
    return status, sw.value


# ------------------------------------------------------------ coverage adjoint (FP64)
def _xf(transform):
    return np.ascontiguousarray(np.asarray(transform, dtype=np.float32))


def adj_forward(rule, ops, w, h, val=None, tolerance=0.3, transform=_abi.IDENTITY):
    """FP64 analytic coverage of one fill: returns (cov, area, status), each (h, w) f64.

    Without `val` the polygon is footile's f32 flattened polygon (the vertices Fig
    receives), widened to double.  With `val` (n_ops x 6 f64) the vertices are the
    Bernstein points of `val` on the subdivision tree the op floats decide (for
    finite differences)."""
    ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
    cov = np.zeros((h, w), np.float64)
    area = np.zeros((h, w), np.float64)
    v = None if val is None else np.ascontiguousarray(val, dtype=np.float64)
    xf = _xf(transform)
    st = lib().orc_adj_forward(rule, _ptr(ops), len(ops), _ptr(v), w, h, tolerance, _ptr(xf), _ptr(cov), _ptr(area))
    return cov, area, st


def adj_backward(rule, ops, w, h, area, grad_cov, val=None, tolerance=0.3, transform=_abi.IDENTITY):
    """FP64 gradient of sum(grad_cov * cov) with respect to the op floats: (n_ops, 6) f64."""
    ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
    area = np.ascontiguousarray(area, dtype=np.float64)
    g = np.ascontiguousarray(grad_cov, dtype=np.float64)
    out = np.zeros((len(ops), 6), np.float64)
    v = None if val is None else np.ascontiguousarray(val, dtype=np.float64)
    xf = _xf(transform)
    lib().orc_adj_backward(rule, _ptr(ops), len(ops), _ptr(v), w, h, tolerance, _ptr(xf), _ptr(area), _ptr(g),
                           _ptr(out))
    return out


def adj_stroke_forward(ops, w, h, val=None, s_width=1.0, tolerance=0.3, transform=_abi.IDENTITY,
                       join=_abi.JOIN_MITER, miter_limit=4.0):
    """FP64 analytic coverage of Plotter::stroke's outline: (cov, area, status).
    With `val` the stroke points are Bernstein points of `val` and widths follow the
    PenWidth values in val[:, 0] (and `s_width`), on the decisions the op floats make."""
    ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
    cov = np.zeros((h, w), np.float64)
    area = np.zeros((h, w), np.float64)
    v = None if val is None else np.ascontiguousarray(val, dtype=np.float64)
    xf = _xf(transform)
    st = lib().orc_adj_stroke_forward(_ptr(ops), len(ops), _ptr(v), s_width, w, h, tolerance, _ptr(xf), join,
                                      miter_limit, _ptr(cov), _ptr(area))
    return cov, area, st


def adj_stroke_backward(ops, w, h, area, grad_cov, val=None, s_width=1.0, tolerance=0.3, transform=_abi.IDENTITY,
                        join=_abi.JOIN_MITER, miter_limit=4.0):
    """FP64 gradient of sum(grad_cov * cov) for a stroke: ((n_ops, 6) op-float gradient,
    with PenWidth ops in column 0, and the gradient for the starting pen width)."""
    ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
    area = np.ascontiguousarray(area, dtype=np.float64)
    g = np.ascontiguousarray(grad_cov, dtype=np.float64)
    out = np.zeros((len(ops), 6), np.float64)
    gsw = ctypes.c_double(0.0)
    v = None if val is None else np.ascontiguousarray(val, dtype=np.float64)
    xf = _xf(transform)
    lib().orc_adj_stroke_backward(_ptr(ops), len(ops), _ptr(v), s_width, w, h, tolerance, _ptr(xf), join, miter_limit,
                                  _ptr(area), _ptr(g), _ptr(out), ctypes.byref(gsw))
    return out, gsw.value


def adj_stroke_outline(ops, s_width=1.0, tolerance=0.3, transform=_abi.IDENTITY, join=_abi.JOIN_MITER,
                       miter_limit=4.0):
    ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
    xf = _xf(transform)
    cap = 1 << 16
    while True:
        out = np.zeros(cap, dtype=_abi.OP_DTYPE)
        n = lib().orc_adj_stroke_outline(_ptr(ops), len(ops), tolerance, _ptr(xf), join, miter_limit, s_width,
                                         _ptr(out), cap)
        if n <= cap:
            return out[:n]
        cap = n


# ------------------------------------------------------------- pixel conversion
def srgb_table():
    """lut[a, c]: straight channel c / a (clamped to 1, 0 at a = 0) through the sRGB
    transfer function (IEC 61966-2-1), rounded to the nearest byte (pix's
    Rgba8p -> SRgba8 step, restated: the pix crate is not vendored)."""
    a = np.arange(256, dtype=np.float64)[:, None]
    c = np.arange(256, dtype=np.float64)[None, :]
    with np.errstate(divide="ignore", invalid="ignore"):
        v = np.minimum(1.0, np.where(a > 0, c / np.maximum(a, 1), 0.0))
    e = np.where(v <= 0.0031308, 12.92 * v, 1.055 * np.power(v, 1.0 / 2.4) - 0.055)
    lut = np.minimum(255.0, np.floor(e * 255.0 + 0.5)).astype(np.uint8)
    lut[0, :] = 0
    return lut


def convert(src):
    """Rgba8p (h, w, 4) -> SRgba8, or Matte8 (h, w) -> SGray8."""
    lut = srgb_table()
    if src.ndim == 3:
        out = src.copy()
        a = src[..., 3]
        for ch in range(3):
            out[..., ch] = lut[a, src[..., ch]]
        return out
    return lut[255, src]


# ------------------------------------------- ordered SrcOver of strokes (FP64 chain)
def adj_stroke_composite(ops, paths, clr, w, h, target, val=None, join=_abi.JOIN_MITER, miter_limit=4.0,
                         tolerance=0.3, transform=_abi.IDENTITY, grads=True, init=None):
    """FP64 loss sum((C_N - target)^2) of strokes SrcOver'd in order on one w x h canvas
    (C_n = clr_n cov_n + C_{n-1} (1 - a_n cov_n), float premultiplied colours, C_0 =
    `init` or 0), and with `grads` its gradient w.r.t. the op floats (n_ops, 6) and the
    starting pen widths (and, with `init`, w.r.t. C_0 as a fifth result).  `val`
    (n_ops x 6) moves the vertices continuously on held decisions (for finite
    differences)."""
    ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
    n = len(paths)
    kw = dict(join=join, miter_limit=miter_limit, tolerance=tolerance, transform=transform)
    covs, areas = [], []
    for p in paths:
        b, k = int(p["op_begin"]), int(p["n_ops"])
        v = None if val is None else val[b:b + k]
        c, a, _ = adj_stroke_forward(ops[b:b + k], w, h, val=v, s_width=float(p["s_width"]), **kw)
        covs.append(c.ravel())
        areas.append(a)
    C = np.zeros((w * h, 4)) if init is None else np.array(init, dtype=np.float64).reshape(w * h, 4)
    C0 = C.copy()
    for i in range(n):
        C = clr[i][None, :] * covs[i][:, None] + C * (1.0 - clr[i][3] * covs[i])[:, None]
    loss = float(((C - target) ** 2).sum())
    if not grads:
        return loss
    G = 2.0 * (C - target)
    # E_{n-1} = G . C_{n-1} forward, then the suffix products backward
    E = (G * C0).sum(axis=1)
    Es = []
    for i in range(n):
        Es.append(E.copy())
        E = (G @ clr[i]) * covs[i] + E * (1.0 - clr[i][3] * covs[i])
    P = np.ones(w * h)
    g_ops = np.zeros((len(ops), 6))
    g_w = np.zeros(n)
    for i in reversed(range(n)):
        gc = P * ((G @ clr[i]) - clr[i][3] * Es[i])
        P = P * (1.0 - clr[i][3] * covs[i])
        p = paths[i]
        b, k = int(p["op_begin"]), int(p["n_ops"])
        v = None if val is None else val[b:b + k]
        gg, gw = adj_stroke_backward(ops[b:b + k], w, h, areas[i], gc.reshape(h, w), val=v,
                                     s_width=float(p["s_width"]), **kw)
        g_ops[b:b + k] += gg
        g_w[i] = gw
    if init is not None:
        return loss, C, g_ops, g_w, G * P[:, None]
    return loss, C, g_ops, g_w
