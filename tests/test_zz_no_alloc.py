"""The allocation-free fill (ft_fill_noalloc) against the context fill (ft_fill) and the
oracle.

ft_fill_noalloc is for hosts that may not allocate device memory, themselves or
through this library: their device memory belongs to another runtime's allocator, or
they run under a fixed device-memory budget.  It keeps its figure scratch in a device
array of the library and takes only inputs and outputs.  Calls in a row on different
paths must each match ft_fill and the oracle bit for bit, so a call never sees the
figure the previous call left in the shared array.  This file is collected last on
purpose, and passes both alone in a fresh process and after every other test.
"""
import ctypes

import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, _lib, workloads
from footile_gb300.path import PathOp, ops_array
from footile_gb300.plotter import Plotter

pytestmark = pytest.mark.gpu


def _noalloc(L):
    fn = L.ft_fill_noalloc
    P = ctypes.c_void_p
    fn.argtypes = [ctypes.c_int32, P, ctypes.c_uint32, ctypes.c_int32, P, P, ctypes.c_uint32, ctypes.c_uint32,
                   ctypes.c_uint32, P, ctypes.c_float, ctypes.c_float, P, P]
    fn.restype = ctypes.c_int
    return fn


def _big_cubics(rng, n, side):
    """`n` cubics spanning the canvas: at tolerance 0.05 one chunk of 256 ops flattens to
    more raw vertices than a shared-memory compaction window holds (2,048), the build's
    re-walked window path."""
    ops = [PathOp.Move(float(rng.random() * side), float(rng.random() * side))]
    for _ in range(n):
        ops.append(PathOp.Cubic(*[float(v) for v in rng.random(6) * side]))
    ops.append(PathOp.Close())
    return ops_array(ops)


# (canvas w, h, rule, tolerance, path builder)
CALLS = [
    (203, 150, _abi.NONZERO, 0.3, lambda rng: workloads.random_path(rng, 203, 50, n_sub=2)),
    (96, 257, _abi.EVENODD, 0.3, lambda rng: workloads.random_path(rng, 257, 80, n_sub=2)),
    (256, 256, _abi.NONZERO, 0.05, lambda rng: _big_cubics(rng, 200, 256)),
]


@pytest.mark.parametrize("fmt", [_abi.MATTE8, _abi.RGBA8P])
def test_noalloc_matches_context_fill_in_a_row(cuda_ok, gpu_lib, fmt):
    torch = pytest.importorskip("torch")
    fill = _noalloc(gpu_lib)
    ctx = _lib.Context(0)
    rng = np.random.default_rng(77)
    bpp = _abi.BYTES_PER_PIXEL[fmt]
    for call, (w, h, rule, tol, make) in enumerate(CALLS):
        ops = make(rng)
        clr = (40, 90, 20, 200)
        shape = (h, w) if fmt == _abi.MATTE8 else (h, w, 4)
        init = rng.integers(0, 256, shape).astype(np.uint8)
        # the context fill (ft_fill) and the oracle
        want = init.copy()
        ctx.set_tolerance(tol)
        ctx.set_pen_width(1.0)
        Plotter(want, context=ctx).fill(rule, ops, clr)
        want_o = init.copy()
        st_o, _ = oracle.fill(rule, ops, want_o, fmt, clr, tolerance=tol)
        assert st_o == _abi.OK
        bad = np.argwhere(want != want_o)
        assert len(bad) == 0, f"call {call}: ft_fill differs from the oracle at {len(bad)} bytes"
        # the allocation-free fill on device buffers
        ops_d = torch.from_numpy(ops.view(np.uint8)).cuda()
        ras_d = torch.from_numpy(init.reshape(h, w * bpp)).cuda()
        st_d = torch.full((1,), -1, dtype=torch.int32, device="cuda")
        c = (ctypes.c_uint8 * 4)(*clr)
        rc = fill(rule, ctypes.c_void_p(ops_d.data_ptr()), len(ops), fmt, c, ctypes.c_void_p(ras_d.data_ptr()), w, h,
                  w * bpp, None, tol, 1.0, ctypes.c_void_p(st_d.data_ptr()),
                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert rc == _abi.OK
        torch.cuda.synchronize()
        assert int(st_d.item()) == _abi.OK
        got = ras_d.cpu().numpy().reshape(shape)
        bad = np.argwhere(got != want)
        assert len(bad) == 0, f"call {call}: {len(bad)} bytes differ from ft_fill, first at {tuple(bad[0])}"
    ctx.close()


def test_noalloc_rejects_too_wide(gpu_lib):
    fill = _noalloc(gpu_lib)
    rc = fill(_abi.NONZERO, None, 0, _abi.MATTE8, None, ctypes.c_void_p(16), _abi.MAX_WIDTH + 1, 1,
              _abi.MAX_WIDTH + 1, None, 0.3, 1.0, None, None)
    assert rc == _abi.ERR_CAP


def test_noalloc_in_a_captured_graph(cuda_ok, gpu_lib):
    """The use the declaration describes: one call made eagerly first (the per-device
    setup), then a call recorded into a CUDA graph during stream capture, replayed onto a
    fresh raster: bit for bit the context fill's raster."""
    torch = pytest.importorskip("torch")
    fill = _noalloc(gpu_lib)
    rng = np.random.default_rng(5)
    clr = (200, 10, 70, 255)
    c = (ctypes.c_uint8 * 4)(*clr)
    s = torch.cuda.Stream()
    warm_ops = torch.from_numpy(workloads.random_path(rng, 64, 20).view(np.uint8)).cuda()
    warm_ras = torch.zeros((64, 64), dtype=torch.uint8, device="cuda")
    rc = fill(_abi.NONZERO, ctypes.c_void_p(warm_ops.data_ptr()), warm_ops.numel() // 32, _abi.MATTE8, c,
              ctypes.c_void_p(warm_ras.data_ptr()), 64, 64, 64, None, 0.3, 1.0, None, ctypes.c_void_p(s.cuda_stream))
    assert rc == _abi.OK
    torch.cuda.synchronize()
    ops = workloads.random_path(rng, 240, 80, n_sub=3)
    ops_d = torch.from_numpy(ops.view(np.uint8)).cuda()
    ras_d = torch.full((240, 240), 9, dtype=torch.uint8, device="cuda")
    st_d = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        rc = fill(_abi.EVENODD, ctypes.c_void_p(ops_d.data_ptr()), len(ops), _abi.MATTE8, c,
                  ctypes.c_void_p(ras_d.data_ptr()), 240, 240, 240, None, 0.3, 1.0,
                  ctypes.c_void_p(st_d.data_ptr()), ctypes.c_void_p(s.cuda_stream))
    assert rc == _abi.OK
    ras_d.fill_(9)
    torch.cuda.synchronize()
    g.replay()
    torch.cuda.synchronize()
    assert int(st_d.item()) == _abi.OK
    ctx = _lib.Context(0)
    want = np.full((240, 240), 9, np.uint8)
    ctx.set_pen_width(1.0)
    Plotter(want, context=ctx).fill(_abi.EVENODD, ops, clr)
    ctx.close()
    got = ras_d.cpu().numpy()
    bad = np.argwhere(got != want)
    assert len(bad) == 0, f"{len(bad)} bytes differ from ft_fill"
