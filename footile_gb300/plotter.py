"""`Plotter` — footile's drawing front end (src/plotter.rs:38-381) over the C ABI.

A Plotter owns a raster and draws paths into it with `fill` / `stroke`, keeping
footile's state between calls: tolerance, transform, join style and the pen
width that `PenWidth` ops leave behind (plotter.rs:151-153).

Rasters:
  * numpy ``uint8`` arrays on the host — shape (h, w) is ``Matte8``,
    shape (h, w, 4) is premultiplied ``Rgba8p``;
  * CUDA tensors (torch) of the same shapes stay on the device (no copies).
"""
import ctypes

import numpy as np

from . import _abi
from ._lib import Context
from .path import FillRule, JoinStyle, ops_array


def _is_torch_cuda(a):
    return type(a).__module__.startswith("torch") and getattr(a, "is_cuda", False)


def raster_format(raster):
    shape = tuple(raster.shape)
    if len(shape) == 2:
        return _abi.MATTE8
    if len(shape) == 3 and shape[2] == 4:
        return _abi.RGBA8P
    raise ValueError("raster must be (h, w) Matte8 or (h, w, 4) Rgba8p uint8")


def _clr_bytes(clr, fmt):
    if clr is None:
        return (ctypes.c_uint8 * 4)(0, 0, 0, 0)
    if np.isscalar(clr):
        v = int(clr)
        return (ctypes.c_uint8 * 4)(v, v, v, v)
    c = [int(v) for v in clr]
    if len(c) == 1:
        c = c * 4
    return (ctypes.c_uint8 * 4)(*c)


class Plotter:
    """src/plotter.rs:38-381.  `Plotter(raster)` takes the raster (plotter.rs:96)."""

    def __init__(self, raster, device=0, context=None):
        self._raster = raster
        self._fmt = raster_format(raster)
        self._ctx = context if context is not None else Context(device)
        self._ops_dev = None

    # -- plotter.rs:118-125
    def width(self):
        return int(self._raster.shape[1])

    def height(self):
        return int(self._raster.shape[0])

    # -- plotter.rs:133-161
    def set_tolerance(self, t):
        self._ctx.set_tolerance(float(t))
        return self

    def set_transform(self, m):
        self._ctx.set_transform(m)
        return self

    def set_join(self, js):
        if not isinstance(js, JoinStyle):
            raise TypeError("set_join takes a JoinStyle")
        self._ctx.set_join(js.kind, js.limit)
        return self

    def pen_width(self):
        """Current pen width (PenWidth ops persist between calls)."""
        return self._ctx.pen_width()

    def context(self):
        return self._ctx

    def _call(self, stroke, rule, ops, clr):
        ops = ops_array(ops) if not _is_torch_cuda(ops) else ops
        r = self._raster
        h, w = int(r.shape[0]), int(r.shape[1])
        c = _clr_bytes(clr, self._fmt)
        L, ctx = self._ctx.L, self._ctx
        if _is_torch_cuda(r):
            import torch
            if not r.is_contiguous() or r.dtype != torch.uint8:
                raise ValueError("device raster must be a contiguous uint8 tensor")
            if _is_torch_cuda(ops):
                ops_ptr, n_ops = ops.data_ptr(), ops.numel() * ops.element_size() // 32
            else:
                t = torch.from_numpy(ops.view(np.uint8)).to(r.device)
                self._ops_dev = t
                ops_ptr, n_ops = t.data_ptr(), len(ops)
            stride = int(r.stride(0)) * r.element_size()
            where, rptr = _abi.DEVICE, ctypes.c_void_p(r.data_ptr())
            optr = ctypes.c_void_p(ops_ptr)
        else:
            if not (isinstance(r, np.ndarray) and r.dtype == np.uint8 and r.flags.c_contiguous):
                raise ValueError("host raster must be a C-contiguous uint8 numpy array")
            n_ops = len(ops)
            stride = int(r.strides[0])
            where = _abi.HOST
            rptr = r.ctypes.data_as(ctypes.c_void_p)
            optr = ops.ctypes.data_as(ctypes.c_void_p)
        if stroke:
            rc = L.ft_stroke(ctx.h, optr, n_ops, self._fmt, c, rptr, w, h, stride, where)
        else:
            rc = L.ft_fill(ctx.h, int(rule), optr, n_ops, self._fmt, c, rptr, w, h, stride, where)
        ctx.check(rc)
        return r

    # -- plotter.rs:339-350
    def fill(self, rule, ops, clr=None):
        return self._call(False, FillRule(rule), ops, clr)

    # -- plotter.rs:356-365
    def stroke(self, ops, clr=None):
        return self._call(True, FillRule.NonZero, ops, clr)

    # -- plotter.rs:368-380
    def raster(self):
        return self._raster

    def raster_mut(self):
        return self._raster

    def into_raster(self):
        r = self._raster
        self._raster = None
        return r


def pack_batch(paths_ops, sizes, fmt=_abi.MATTE8, clrs=None, s_width=1.0):
    """Pack per-path op arrays and square/rect canvas sizes into one batch.

    Returns (ops, paths, raster_bytes): all ops concatenated, the `ft_path_desc`
    array, and the size of one buffer holding every raster back to back (rows
    padded to 4 bytes).
    """
    bpp = _abi.BYTES_PER_PIXEL[fmt]
    n = len(paths_ops)
    paths = np.zeros(n, dtype=_abi.PATH_DTYPE)
    lens = np.array([len(o) for o in paths_ops], dtype=np.int64)
    begins = np.concatenate([[0], np.cumsum(lens)[:-1]]) if n else np.zeros(0, np.int64)
    off = 0
    for i, (o, sz) in enumerate(zip(paths_ops, sizes)):
        w, h = (sz, sz) if np.isscalar(sz) else sz
        stride = ((w * bpp + 3) // 4) * 4
        paths[i]["op_begin"] = begins[i]
        paths[i]["n_ops"] = lens[i]
        paths[i]["width"] = w
        paths[i]["height"] = h
        paths[i]["raster_offset"] = off
        paths[i]["stride"] = stride
        paths[i]["s_width"] = s_width
        if clrs is not None:
            paths[i]["clr"] = clrs[i]
        off += stride * h
    ops = ops_array(paths_ops) if n else np.zeros(0, dtype=_abi.OP_DTYPE)
    return ops, paths, off


def fill_batch(ctx, ops, paths, fmt, rasters, rule=FillRule.NonZero, stroke=False):
    """One persistent launch over many independent Plotter calls (`ft_fill_batch`).

    `ops` / `rasters` are host numpy arrays (copied in and out; Matte8 rasters in
    page-locked memory, e.g. a pinned torch tensor's `.numpy()`, are written in place by
    the kernels) or CUDA tensors (device-resident, asynchronous).  `paths` is a host
    `ft_path_desc` array.
    Returns the per-path status array.
    """
    paths = np.ascontiguousarray(paths, dtype=_abi.PATH_DTYPE)
    if _is_torch_cuda(rasters):
        where = _abi.DEVICE
        ctx.torch_fence()
        optr, n_ops = ops.data_ptr(), ops.numel() * ops.element_size() // 32
        rptr, nbytes = rasters.data_ptr(), rasters.numel() * rasters.element_size()
    else:
        where = _abi.HOST
        ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
        optr, n_ops = ops.ctypes.data, len(ops)
        rptr, nbytes = rasters.ctypes.data, rasters.nbytes
    rc = ctx.L.ft_fill_batch(ctx.h, int(bool(stroke)), int(rule), ctypes.c_void_p(optr), n_ops,
                             paths.ctypes.data_as(ctypes.c_void_p), len(paths), fmt, ctypes.c_void_p(rptr),
                             nbytes, where)
    ctx.check(rc)
    return ctx.batch_status(len(paths))


class PreparedBatch:
    """A batch planned once (`ft_batch_create`) and launched many times from a CUDA
    graph (`ft_batch_launch`) on device-resident ops and rasters."""

    def __init__(self, ctx, paths, fmt=_abi.MATTE8, rule=FillRule.NonZero, stroke=False):
        self.ctx = ctx
        self.paths = np.ascontiguousarray(paths, dtype=_abi.PATH_DTYPE)
        self.n = len(self.paths)
        h = ctypes.c_void_p()
        ctx.check(ctx.L.ft_batch_create(ctx.h, int(bool(stroke)), int(rule),
                                        self.paths.ctypes.data_as(ctypes.c_void_p), self.n, fmt, ctypes.byref(h)))
        self.h = h

    def launch(self, ops_dev, rasters_dev):
        """Asynchronous launch on the context stream (CUDA tensors or raw pointers)."""
        if hasattr(ops_dev, "data_ptr"):
            optr, n_ops = ops_dev.data_ptr(), ops_dev.numel() * ops_dev.element_size() // 32
            rptr, nbytes = rasters_dev.data_ptr(), rasters_dev.numel() * rasters_dev.element_size()
        else:
            (optr, n_ops), (rptr, nbytes) = ops_dev, rasters_dev
        self.ctx.check(self.ctx.L.ft_batch_launch(self.ctx.h, self.h, ctypes.c_void_p(optr), n_ops,
                                                  ctypes.c_void_p(rptr), nbytes))

    def status(self):
        st = np.zeros(self.n, dtype=np.int32)
        self.ctx.check(self.ctx.L.ft_batch_launch_status(self.ctx.h, self.h, st.ctypes.data_as(ctypes.c_void_p),
                                                         self.n))
        return st

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.ft_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pen_width_chain(ops, paths, s_width=1.0):
    """Pen width at the start of each call of a sequence of Plotter calls: footile
    keeps the last PenWidth from call to call (plotter.rs:151-153)."""
    ops = np.asarray(ops, dtype=_abi.OP_DTYPE)
    out = np.empty(len(paths), np.float32)
    pw = np.flatnonzero(ops["kind"] == _abi.OP_PEN_WIDTH)
    cur = np.float32(s_width)
    for i, d in enumerate(paths):
        out[i] = cur
        b, n = int(d["op_begin"]), int(d["n_ops"])
        k = np.searchsorted(pw, b + n) - 1
        if k >= 0 and pw[k] >= b:
            cur = ops["v"][pw[k], 0]
    return out, cur


def composite_batch(ctx, ops, paths, fmt, raster, rule=FillRule.NonZero, stroke=False, s_width=None):
    """Draw every path onto one raster in order (`ft_composite_batch`), as a
    sequence of Plotter::fill / Plotter::stroke calls on one Plotter would.

    `raster` is an (h, w) Matte8 or (h, w, 4) Rgba8p numpy array (host) or CUDA
    tensor (device).  Path colours come from `paths["clr"]`.  With host ops the pen
    width chain is computed here, starting from the context's pen width (or
    `s_width`); the context's pen width is left at the sequence's final value.
    Returns the per-path status array."""
    paths = np.array(paths, dtype=_abi.PATH_DTYPE)
    h, w = int(raster.shape[0]), int(raster.shape[1])
    if _is_torch_cuda(raster):
        where = _abi.DEVICE
        ctx.torch_fence()
        optr, n_ops = ops.data_ptr(), ops.numel() * ops.element_size() // 32
        rptr = raster.data_ptr()
        stride = int(raster.stride(0)) * raster.element_size()
    else:
        where = _abi.HOST
        ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
        optr, n_ops = ops.ctypes.data, len(ops)
        rptr = raster.ctypes.data
        stride = int(raster.strides[0])
        start = ctx.pen_width() if s_width is None else s_width
        paths["s_width"], last = pen_width_chain(ops, paths, start)
        ctx.set_pen_width(float(last))
    rc = ctx.L.ft_composite_batch(ctx.h, int(bool(stroke)), int(rule), ctypes.c_void_p(optr), n_ops,
                                  paths.ctypes.data_as(ctypes.c_void_p), len(paths), fmt, ctypes.c_void_p(rptr),
                                  w, h, stride, where)
    ctx.check(rc)
    return ctx.batch_status(len(paths))
