"""ctypes binding of libfootile_gpu.so (the C ABI in include/footile_gpu.h).

The library is built in-tree by `footile_gb300._build`.  There is no CPU
fallback: if the shared library is missing or no GPU is present, every call
raises.
"""
import ctypes
import os
import threading

from . import _abi
from ._build import LIB, build, up_to_date

_lock = threading.Lock()
_lib = None


class FootileError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_abi.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def load(auto_build=True, path=None):
    """Load libfootile_gpu.so, compiling it first when it is missing or stale.  `path`
    loads another build of the library instead (the bounds-check build of the tests);
    it must come before the first load of the process."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if path is None and not up_to_date():
            if not auto_build:
                raise RuntimeError(f"{LIB} is missing; run footile_gb300._build.build()")
            build()
        L = ctypes.CDLL(path or LIB)
        P = ctypes.c_void_p
        i32, u32, u64, f32 = ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_float
        sig = {
            "ft_ctx_create": ([ctypes.c_int, ctypes.POINTER(P)], ctypes.c_int),
            "ft_ctx_destroy": ([P], None),
            "ft_set_stream": ([P, P], ctypes.c_int),
            "ft_set_tolerance": ([P, f32], ctypes.c_int),
            "ft_set_transform": ([P, P], ctypes.c_int),
            "ft_set_join": ([P, i32, f32], ctypes.c_int),
            "ft_set_pen_width": ([P, f32], ctypes.c_int),
            "ft_get_pen_width": ([P, ctypes.POINTER(f32)], ctypes.c_int),
            "ft_set_figure_cap": ([P, u32], ctypes.c_int),
            "ft_get_figure_cap": ([P, ctypes.POINTER(u32)], ctypes.c_int),
            "ft_fill": ([P, i32, P, u32, i32, P, P, u32, u32, u32, i32], ctypes.c_int),
            "ft_stroke": ([P, P, u32, i32, P, P, u32, u32, u32, i32], ctypes.c_int),
            "ft_fill_batch": ([P, i32, i32, P, u32, P, u32, i32, P, u64, i32], ctypes.c_int),
            "ft_batch_status": ([P, P, u32], ctypes.c_int),
            "ft_sync": ([P], ctypes.c_int),
            "ft_last_error": ([P], ctypes.c_char_p),
            "ft_last_timings": ([P, ctypes.POINTER(f32)], ctypes.c_int),
            "ft_last_composite_ms": ([P, ctypes.POINTER(f32)], ctypes.c_int),
            "ft_check_failures": ([P, P], ctypes.c_int),
            "ft_launch_count": ([P], u64),
            "ft_batch_create": ([P, i32, i32, P, u32, i32, ctypes.POINTER(P)], ctypes.c_int),
            "ft_batch_launch": ([P, P, P, u32, P, u64], ctypes.c_int),
            "ft_batch_launch_status": ([P, P, P, u32], ctypes.c_int),
            "ft_batch_destroy": ([P], None),
            "ft_composite_batch": ([P, i32, i32, P, u32, P, u32, i32, P, u32, u32, u32, i32], ctypes.c_int),
            "ft_adjoint_forward": ([P, i32, i32, P, u32, P, u32, P, u64, i32, ctypes.POINTER(P)], ctypes.c_int),
            "ft_adjoint_backward": ([P, P, P, P, P, i32], ctypes.c_int),
            "ft_adjoint_status": ([P, P, P, u32], ctypes.c_int),
            "ft_adjoint_destroy": ([P], None),
            "ft_set_tuning": ([P, P], ctypes.c_int),
            "ft_convert": ([P, i32, P, u32, i32, P, u32, u32, u32, i32], ctypes.c_int),
            "ft_srcover_forward": ([P, P, u32, u64, P, P, P, u32], ctypes.c_int),
            "ft_srcover_backward": ([P, P, u32, u64, P, P, P, P, P, u32], ctypes.c_int),
            "ft_stroke_composite_forward": ([P, P, u32, P, u32, P, u32, u32, P, P, u32, i32, ctypes.POINTER(P)],
                                            ctypes.c_int),
            "ft_stroke_composite_backward": ([P, P, P, P, P, P, i32], ctypes.c_int),
            "ft_stroke_composite_status": ([P, P, P, u32], ctypes.c_int),
            "ft_stroke_composite_chunk": ([P], u32),
            "ft_stroke_composite_destroy": ([P], None),
            "ft_get_tuning": ([P, P], ctypes.c_int),
            "ft_autotune_batch": ([P, i32, i32, P, u32, P, u32, i32, P, u64, ctypes.c_char_p, P,
                                   ctypes.POINTER(f32)], ctypes.c_int),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
        return _lib


def exported_symbols():
    """Names of the C ABI functions declared in include/footile_gpu.h."""
    return [n for n in (
        "ft_ctx_create", "ft_ctx_destroy", "ft_set_stream", "ft_set_tolerance", "ft_set_transform",
        "ft_set_join", "ft_set_pen_width", "ft_get_pen_width", "ft_fill", "ft_stroke", "ft_fill_batch",
        "ft_batch_status", "ft_sync", "ft_last_error", "ft_last_timings", "ft_last_composite_ms", "ft_launch_count",
        "ft_check_failures",
        "ft_batch_create", "ft_batch_launch", "ft_batch_launch_status", "ft_batch_destroy",
        "ft_composite_batch", "ft_fill_noalloc", "ft_adjoint_forward", "ft_adjoint_backward", "ft_adjoint_status",
        "ft_adjoint_destroy", "ft_set_tuning", "ft_get_tuning", "ft_autotune_batch",
        "ft_convert", "ft_srcover_forward", "ft_srcover_backward", "ft_stroke_composite_forward",
        "ft_stroke_composite_backward", "ft_stroke_composite_status", "ft_stroke_composite_chunk",
        "ft_stroke_composite_destroy", "ft_set_figure_cap", "ft_get_figure_cap")]


class Tuning(ctypes.Structure):
    """`ft_tuning`: the knobs of a batch plan (see include/footile_gpu.h)."""
    _fields_ = [("warp_max_side", ctypes.c_int32), ("cta_smem_bytes", ctypes.c_int32),
                ("split_px", ctypes.c_int32), ("grid_per_sm", ctypes.c_int32), ("band_rows", ctypes.c_int32),
                ("pool_edges", ctypes.c_int32), ("host_chunks", ctypes.c_int32), ("host_mapped", ctypes.c_int32),
                ("tile_w", ctypes.c_int32), ("tile_stage", ctypes.c_int32),
                ("fig_build", ctypes.c_int32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class Context:
    """One `ft_ctx`: footile's Plotter settings plus device buffers and a stream."""

    def __init__(self, device=0):
        self.L = load()
        h = ctypes.c_void_p()
        rc = self.L.ft_ctx_create(device, ctypes.byref(h))
        if rc != _abi.OK:
            raise FootileError(rc, "ft_ctx_create failed (no usable CUDA device?)")
        self.h = h
        self.stream_ptr = None  # the context's own stream until set_stream

    def close(self):
        if getattr(self, "h", None):
            self.L.ft_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc):
        if rc != _abi.OK:
            raise FootileError(rc, self.L.ft_last_error(self.h).decode())
        return rc

    def set_tolerance(self, t):
        self.check(self.L.ft_set_tolerance(self.h, t))

    def set_transform(self, m):
        arr = (ctypes.c_float * 6)(*[float(v) for v in m])
        self.check(self.L.ft_set_transform(self.h, arr))

    def set_join(self, kind, limit):
        self.check(self.L.ft_set_join(self.h, kind, limit))

    def set_pen_width(self, w):
        self.check(self.L.ft_set_pen_width(self.h, w))

    def set_figure_cap(self, max_points):
        """Un-capped figures (a documented extension): fills keep up to `max_points`
        vertices per figure; 0 restores footile's 65,535 (`ft_set_figure_cap`)."""
        self.check(self.L.ft_set_figure_cap(self.h, int(max_points)))

    def figure_cap(self):
        v = ctypes.c_uint32()
        self.check(self.L.ft_get_figure_cap(self.h, ctypes.byref(v)))
        return v.value

    def pen_width(self):
        v = ctypes.c_float()
        self.check(self.L.ft_get_pen_width(self.h, ctypes.byref(v)))
        return v.value

    def set_stream(self, stream_ptr):
        self.check(self.L.ft_set_stream(self.h, ctypes.c_void_p(stream_ptr)))
        self.stream_ptr = int(stream_ptr)

    def torch_fence(self):
        """Order a call on CUDA tensors after the work torch has queued for them: a
        no-op when the context runs on torch's current stream, otherwise the host
        waits for that stream.  Returns True when the caller must also wait for the
        context (`sync`) before torch reads the results."""
        import torch
        cur = torch.cuda.current_stream()
        if self.stream_ptr == int(cur.cuda_stream):
            return False
        cur.synchronize()
        return True

    def sync(self):
        self.check(self.L.ft_sync(self.h))

    def last_ms(self):
        v = ctypes.c_float()
        self.check(self.L.ft_last_timings(self.h, ctypes.byref(v)))
        return v.value

    def last_composite_ms(self):
        """Device time of the last call's Rgba8p tile compositor alone (0 if it did not run)."""
        v = ctypes.c_float()
        self.check(self.L.ft_last_composite_ms(self.h, ctypes.byref(v)))
        return v.value

    def launch_count(self):
        return int(self.L.ft_launch_count(self.h))

    def set_tuning(self, tuning=None):
        """Set the plan knobs from a dict (or `Tuning`); None restores the defaults."""
        if tuning is None:
            self.check(self.L.ft_set_tuning(self.h, None))
            return
        t = tuning if isinstance(tuning, Tuning) else Tuning(**tuning)
        self.check(self.L.ft_set_tuning(self.h, ctypes.byref(t)))

    def tuning(self):
        t = Tuning()
        self.check(self.L.ft_get_tuning(self.h, ctypes.byref(t)))
        return t.as_dict()

    def tune(self, **knobs):
        """Change some plan knobs, keeping the others as they are in effect."""
        t = self.tuning()
        t.update(knobs)
        self.set_tuning(t)

    def autotune(self, ops_dev, paths, fmt, rasters_dev, rule=0, stroke=False, cache_path=None):
        """Time candidate plans of a batch on device buffers (CUDA tensors) and keep the
        fastest as this context's tuning.  Returns (tuning dict, ms or 0 from the cache)."""
        import numpy as np
        paths = np.ascontiguousarray(paths, dtype=_abi.PATH_DTYPE)
        n_ops = ops_dev.numel() * ops_dev.element_size() // 32
        nbytes = rasters_dev.numel() * rasters_dev.element_size()
        t = Tuning()
        ms = ctypes.c_float()
        cp = cache_path.encode() if cache_path else None
        self.check(self.L.ft_autotune_batch(self.h, int(bool(stroke)), int(rule), ctypes.c_void_p(ops_dev.data_ptr()),
                                            n_ops, paths.ctypes.data_as(ctypes.c_void_p), len(paths), fmt,
                                            ctypes.c_void_p(rasters_dev.data_ptr()), nbytes, cp, ctypes.byref(t),
                                            ctypes.byref(ms)))
        return t.as_dict(), ms.value

    def convert(self, src, dst):
        """Rgba8p (h, w, 4) -> SRgba8, or Matte8 (h, w) -> SGray8 (`ft_convert`): numpy
        arrays (host) or CUDA tensors (device); `dst` may be `src`.  Returns `dst`."""
        dev = hasattr(src, "data_ptr")
        rgba = (src.dim() if dev else src.ndim) == 3
        h, w = int(src.shape[0]), int(src.shape[1])
        if dev:
            wait = self.torch_fence()
            sp, ss = src.data_ptr(), int(src.stride(0)) * src.element_size()
            dp, ds = dst.data_ptr(), int(dst.stride(0)) * dst.element_size()
        else:
            sp, ss = src.ctypes.data, int(src.strides[0])
            dp, ds = dst.ctypes.data, int(dst.strides[0])
        self.check(self.L.ft_convert(self.h, _abi.RGBA8P if rgba else _abi.MATTE8, ctypes.c_void_p(sp), ss,
                                     _abi.SRGBA8 if rgba else _abi.SGRAY8, ctypes.c_void_p(dp), ds, w, h,
                                     _abi.DEVICE if dev else _abi.HOST))
        if dev and wait:
            self.sync()
        return dst

    def batch_status(self, n):
        import numpy as np
        st = np.zeros(n, dtype=np.int32)
        self.check(self.L.ft_batch_status(self.h, st.ctypes.data_as(ctypes.c_void_p), n))
        return st
