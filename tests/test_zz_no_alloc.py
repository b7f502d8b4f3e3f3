"""The allocation-free fill (ft_fill_noalloc) against the context fill (ft_fill).

ft_fill_noalloc serves callers that cannot allocate device memory (work captured
into a CUDA graph, fixed memory budgets, foreign device allocators): it keeps its
scratch in a device array of the library and takes only inputs and outputs.
Two calls in a row on different paths must each match ft_fill bit for bit, so a
call never sees the previous call's scratch.  Collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from footile_gb300 import _abi, _lib, workloads
from footile_gb300.plotter import Plotter

pytestmark = pytest.mark.gpu


def _noalloc(L):
    fn = L.ft_fill_noalloc
    P = ctypes.c_void_p
    fn.argtypes = [ctypes.c_int32, P, ctypes.c_uint32, ctypes.c_int32, P, P, ctypes.c_uint32, ctypes.c_uint32,
                   ctypes.c_uint32, P, ctypes.c_float, ctypes.c_float, P, P]
    fn.restype = ctypes.c_int
    return fn


@pytest.mark.parametrize("fmt", [_abi.MATTE8, _abi.RGBA8P])
def test_noalloc_matches_context_fill_twice(cuda_ok, gpu_lib, fmt):
    torch = pytest.importorskip("torch")
    fill = _noalloc(gpu_lib)
    ctx = _lib.Context(0)
    rng = np.random.default_rng(77)
    bpp = _abi.BYTES_PER_PIXEL[fmt]
    for call in range(2):
        w, h = (203, 150) if call == 0 else (96, 257)
        ops = workloads.random_path(rng, max(w, h), 50 + 30 * call, n_sub=2)
        rule = _abi.NONZERO if call == 0 else _abi.EVENODD
        clr = (40, 90, 20, 200)
        init = rng.integers(0, 256, (h, w * bpp)).astype(np.uint8)
        want = init.copy().reshape((h, w) if fmt == _abi.MATTE8 else (h, w, 4))
        Plotter(want, context=ctx).fill(rule, ops, clr)
        ops_d = torch.from_numpy(ops.view(np.uint8)).cuda()
        ras_d = torch.from_numpy(init).cuda()
        st_d = torch.full((1,), -1, dtype=torch.int32, device="cuda")
        c = (ctypes.c_uint8 * 4)(*clr)
        rc = fill(rule, ctypes.c_void_p(ops_d.data_ptr()), len(ops), fmt, c, ctypes.c_void_p(ras_d.data_ptr()), w, h,
                  w * bpp, None, 0.3, 1.0, ctypes.c_void_p(st_d.data_ptr()),
                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert rc == _abi.OK
        torch.cuda.synchronize()
        assert int(st_d.item()) == _abi.OK
        got = ras_d.cpu().numpy().reshape(want.shape)
        bad = np.argwhere(got != want)
        assert len(bad) == 0, f"call {call}: {len(bad)} bytes differ, first at {tuple(bad[0])}"
    ctx.close()


def test_noalloc_rejects_too_wide(gpu_lib):
    fill = _noalloc(gpu_lib)
    rc = fill(_abi.NONZERO, None, 0, _abi.MATTE8, None, ctypes.c_void_p(16), _abi.MAX_WIDTH + 1, 1,
              _abi.MAX_WIDTH + 1, None, 0.3, 1.0, None, None)
    assert rc == _abi.ERR_CAP
