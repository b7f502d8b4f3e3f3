"""Coverage adjoint: the differentiable FP32 coverage of a batch of fills
(`ft_adjoint_forward` / `ft_adjoint_backward` in include/footile_gpu.h).

footile has no gradients; this is the path's differentiable companion.  The
coverage of each path is the exact area of its flattened polygon in every pixel
(footile's pen walk and De Casteljau subdivision, plotter.rs:175-332; the cell-area
scheme of fig.rs:285-321 without the fixed-point quantisation; NonZero / EvenOdd as
in imgbuf.rs:38-199), and the backward gives d(loss)/d(op floats) with the
subdivision tree held fixed, recomputing the flattened edges instead of storing
them.  `CoverageFn` wraps the pair as a `torch.autograd.Function`.
"""
import ctypes

import numpy as np

from . import _abi
from ._lib import Context, load


def pack_coverage(paths_ops, sizes, s_width=1.0):
    """Pack per-path op arrays and canvas sizes: (ops, paths, cov_bytes), one f32
    coverage plane per path, back to back (row stride 4 * width); every path starts
    with pen width `s_width` (footile's default 1.0)."""
    n = len(paths_ops)
    paths = np.zeros(n, dtype=_abi.PATH_DTYPE)
    lens = np.array([len(o) for o in paths_ops], dtype=np.int64)
    begins = np.concatenate([[0], np.cumsum(lens)[:-1]]) if n else np.zeros(0, np.int64)
    off = 0
    for i, sz in enumerate(sizes):
        w, h = (sz, sz) if np.isscalar(sz) else sz
        paths[i]["op_begin"] = begins[i]
        paths[i]["n_ops"] = lens[i]
        paths[i]["width"] = w
        paths[i]["height"] = h
        paths[i]["raster_offset"] = off
        paths[i]["stride"] = 4 * w
        paths[i]["s_width"] = s_width
        off += 4 * w * h
    ops = np.concatenate([np.ascontiguousarray(o, dtype=_abi.OP_DTYPE) for o in paths_ops]) if n else \
        np.zeros(0, dtype=_abi.OP_DTYPE)
    return ops, paths, off


def _ptr(x):
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return ctypes.c_void_p(x.data_ptr())
    return x.ctypes.data_as(ctypes.c_void_p)


class Adjoint:
    """Saved state of one forward (`ft_adjoint*`), reusable across calls."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.h = ctypes.c_void_p()
        self.n_ops = 0
        self.n_paths = 0

    def forward(self, rule, ops, paths, cov, stroke=False):
        """Coverage of every path into `cov` (numpy f32 array, or a CUDA tensor with
        `ops` a CUDA tensor of ft_op records); returns `cov`.  With `stroke` the paths are
        stroked (context join, paths["s_width"] as starting pen width).  CUDA tensors
        are used on the context's stream, ordered after torch's current stream
        (Context.torch_fence)."""
        paths = np.ascontiguousarray(paths, dtype=_abi.PATH_DTYPE)
        dev = hasattr(cov, "data_ptr")
        where = _abi.DEVICE if dev else _abi.HOST
        if dev:
            n_ops = ops.numel() * ops.element_size() // 32
        else:
            ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
            n_ops = len(ops)
        nbytes = cov.numel() * 4 if dev else cov.nbytes
        wait = self.ctx.torch_fence() if dev else False
        self.ctx.check(self.ctx.L.ft_adjoint_forward(self.ctx.h, int(bool(stroke)), int(rule), _ptr(ops), n_ops,
                                                     _ptr(paths), len(paths), _ptr(cov), nbytes, where,
                                                     ctypes.byref(self.h)))
        self.n_ops, self.n_paths = n_ops, len(paths)
        if wait:
            self.ctx.sync()
        return cov

    def backward(self, grad_cov, grad_ops, grad_width=None):
        """d(loss)/d(op floats) into `grad_ops` ((n_ops, 6) f32), given d(loss)/d(cov)."""
        dev = hasattr(grad_cov, "data_ptr")
        where = _abi.DEVICE if dev else _abi.HOST
        wait = self.ctx.torch_fence() if dev else False
        self.ctx.check(self.ctx.L.ft_adjoint_backward(self.ctx.h, self.h, _ptr(grad_cov), _ptr(grad_ops),
                                                      _ptr(grad_width), where))
        if wait:
            self.ctx.sync()
        return grad_ops

    def status(self):
        st = np.zeros(self.n_paths, dtype=np.int32)
        self.ctx.check(self.ctx.L.ft_adjoint_status(self.ctx.h, self.h, _ptr(st), self.n_paths))
        return st

    def close(self):
        if self.h:
            load().ft_adjoint_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ops_tensor(kinds, ctrl):
    """Device `ft_op` records (n, 8 f32 words) from op kinds (n int32) and op floats ctrl (n, 6)."""
    import torch
    n = ctrl.shape[0]
    rec = torch.zeros((n, 8), dtype=torch.float32, device=ctrl.device)
    rec[:, 0] = torch.as_tensor(np.asarray(kinds, dtype=np.int32)).to(ctrl.device).view(torch.float32)
    rec[:, 1:7] = ctrl.detach()
    return rec


def make_coverage_fn():
    """A `torch.autograd.Function`: coverage = CoverageFn.apply(ctrl, kinds, paths, cov_numel, rule, adjoint)."""
    import torch

    class CoverageFn(torch.autograd.Function):
        @staticmethod
        def forward(fctx, ctrl, kinds, paths, cov_numel, rule, adj):
            rec = ops_tensor(kinds, ctrl)
            cov = torch.empty(cov_numel, dtype=torch.float32, device=ctrl.device)
            adj.forward(rule, rec, paths, cov)
            fctx.adj = adj
            fctx.n_ops = ctrl.shape[0]
            return cov

        @staticmethod
        def backward(fctx, grad_cov):
            g = torch.empty((fctx.n_ops, 6), dtype=torch.float32, device=grad_cov.device)
            fctx.adj.backward(grad_cov.contiguous(), g)
            return g, None, None, None, None, None

    return CoverageFn


# ------------------------------------------------------- ordered SrcOver adjoint
def srcover_forward(ctx, cov, n_layers, plane, clr, out, init=None):
    """C_N of the ordered SrcOver of `n_layers` coverage planes (`ft_srcover_forward`).
    CUDA tensors: cov (n_layers * plane floats), clr (n_layers x 4 premultiplied
    float), out / init (n_px x 4 float).  Returns `out`."""
    wait = ctx.torch_fence()
    ctx.check(ctx.L.ft_srcover_forward(ctx.h, _ptr(cov), n_layers, plane, _ptr(clr), _ptr(init), _ptr(out),
                                       out.shape[0]))
    if wait:
        ctx.sync()
    return out


def srcover_backward(ctx, cov, n_layers, plane, clr, grad_out, grad_cov, init=None, grad_init=None):
    """dLoss/dcov of every layer (and dLoss/dC_0) from dLoss/dC_N (`ft_srcover_backward`)."""
    wait = ctx.torch_fence()
    ctx.check(ctx.L.ft_srcover_backward(ctx.h, _ptr(cov), n_layers, plane, _ptr(clr), _ptr(init), _ptr(grad_out),
                                        _ptr(grad_cov), _ptr(grad_init), grad_out.shape[0]))
    if wait:
        ctx.sync()
    return grad_cov


class StrokeComposite:
    """Saved state of the differentiable ordered composite of strokes on one canvas
    (`ft_stroke_composite_forward` / `ft_stroke_composite_backward`): the strokes are
    covered in chunks, only the canvas before each chunk is kept, and the backward
    recomputes coverage chunk by chunk.  Numpy arrays or CUDA tensors (all alike)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.h = ctypes.c_void_p()
        self.n_paths = 0

    def forward(self, ops, paths, clr, width, height, out, init=None, chunk=0):
        """C_N of the strokes `paths` (op ranges and starting pen widths) SrcOver'd in
        order with premultiplied colours `clr` ((n, 4) f32) on a width x height canvas
        starting at `init` ((w*h, 4) f32, None: 0), into `out` ((w*h, 4) f32)."""
        paths = np.ascontiguousarray(paths, dtype=_abi.PATH_DTYPE)
        dev = hasattr(out, "data_ptr")
        if dev:
            n_ops = ops.numel() * ops.element_size() // 32
        else:
            ops = np.ascontiguousarray(ops, dtype=_abi.OP_DTYPE)
            clr = np.ascontiguousarray(clr, dtype=np.float32)
            init = None if init is None else np.ascontiguousarray(init, dtype=np.float32)
            n_ops = len(ops)
        wait = self.ctx.torch_fence() if dev else False
        self.ctx.check(self.ctx.L.ft_stroke_composite_forward(
            self.ctx.h, _ptr(ops), n_ops, _ptr(paths), len(paths), _ptr(clr), int(width), int(height), _ptr(init),
            _ptr(out), int(chunk), _abi.DEVICE if dev else _abi.HOST, ctypes.byref(self.h)))
        self.n_paths = len(paths)
        if wait:
            self.ctx.sync()
        return out

    def backward(self, grad_out, grad_ops, grad_width=None, grad_init=None):
        """dLoss/d(op floats) into `grad_ops` ((n_ops, 6) f32), dLoss/d(starting pen
        width) into `grad_width` and dLoss/dC_0 into `grad_init`, given dLoss/dC_N."""
        dev = hasattr(grad_out, "data_ptr")
        wait = self.ctx.torch_fence() if dev else False
        self.ctx.check(self.ctx.L.ft_stroke_composite_backward(
            self.ctx.h, self.h, _ptr(grad_out), _ptr(grad_ops), _ptr(grad_width), _ptr(grad_init),
            _abi.DEVICE if dev else _abi.HOST))
        if wait:
            self.ctx.sync()
        return grad_ops

    @property
    def chunk(self):
        return int(self.ctx.L.ft_stroke_composite_chunk(self.h))

    def status(self):
        st = np.zeros(self.n_paths, dtype=np.int32)
        self.ctx.check(self.ctx.L.ft_stroke_composite_status(self.ctx.h, self.h, _ptr(st), self.n_paths))
        return st

    def close(self):
        if self.h:
            load().ft_stroke_composite_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def stroke_composite_grads(ctx, ops_dev, paths, clr_dev, width, height, target_dev, comp=None, chunk=0):
    """Forward and backward of the differentiable ordered composite of strokes on one
    canvas (StrokeComposite), loss sum((C_N - target)^2): the gradients of the op floats
    (PenWidth ops in column 0) and of the starting pen widths.  Device tensors.  Returns
    (loss, C_N, grad_ops, grad_width, timings in ms)."""
    import torch
    dev = ops_dev.device
    comp = comp or StrokeComposite(ctx)
    out = torch.empty((width * height, 4), dtype=torch.float32, device=dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    stream = torch.cuda.current_stream(dev)
    ev[0].record(stream)
    comp.forward(ops_dev, paths, clr_dev, width, height, out, chunk=chunk)
    ev[1].record(stream)
    g_out = 2.0 * (out - target_dev)
    loss = ((out - target_dev) ** 2).sum()
    g_ops = torch.empty((ops_dev.numel() * ops_dev.element_size() // 32, 6), dtype=torch.float32, device=dev)
    g_w = torch.empty(len(paths), dtype=torch.float32, device=dev)
    ev[2].record(stream)
    comp.backward(g_out, g_ops, g_w)
    ev[3].record(stream)
    torch.cuda.synchronize()
    ms = {"fwd_ms": ev[0].elapsed_time(ev[1]), "bwd_ms": ev[2].elapsed_time(ev[3]), "chunk": comp.chunk}
    return loss, out, g_ops, g_w, ms
