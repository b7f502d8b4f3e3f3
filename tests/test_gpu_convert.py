"""ft_convert on the GPU against the oracle's table, byte for byte: vector and tail
paths, padded strides, host and device buffers, in place."""
import numpy as np
import pytest

import oracle
from footile_gb300 import _abi
from footile_gb300._lib import FootileError

pytestmark = pytest.mark.gpu


def premul(rng, h, w):
    a = rng.integers(0, 256, (h, w)).astype(np.uint8)
    rgb = (rng.random((h, w, 3)) * (a[..., None].astype(np.float64) + 1)).clip(0, 255).astype(np.uint8)
    return np.ascontiguousarray(np.concatenate([rgb, a[..., None]], axis=2))


@pytest.mark.parametrize("w,h", [(256, 256), (203, 37), (1, 1), (4, 3), (1000, 7)])
def test_rgba_host(ctx, w, h):
    src = premul(np.random.default_rng(w * 7 + h), h, w)
    dst = np.zeros_like(src)
    ctx.convert(src, dst)
    assert np.array_equal(dst, oracle.convert(src))


@pytest.mark.parametrize("w,h", [(256, 256), (203, 37), (33, 5)])
def test_matte_host(ctx, w, h):
    src = np.random.default_rng(w + h).integers(0, 256, (h, w)).astype(np.uint8)
    dst = np.zeros_like(src)
    ctx.convert(src, dst)
    assert np.array_equal(dst, oracle.convert(src))


def test_device_padded_and_in_place(ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    src = premul(rng, 64, 100)
    big = np.zeros((64, 128, 4), np.uint8)  # padded rows: stride 512 bytes, width 100
    big[:, :100] = src
    t = torch.from_numpy(big).cuda()
    view = t[:, :100]
    ctx.convert(view, view)  # in place
    got = t.cpu().numpy()
    assert np.array_equal(got[:, :100], oracle.convert(src))
    assert not got[:, 100:].any()
    m = torch.from_numpy(rng.integers(0, 256, (2048, 2048)).astype(np.uint8)).cuda()
    out = torch.empty_like(m)
    ctx.convert(m, out)
    assert np.array_equal(out.cpu().numpy(), oracle.convert(m.cpu().numpy()))


def test_bad_formats(ctx):
    src = np.zeros((4, 4), np.uint8)
    import ctypes
    rc = ctx.L.ft_convert(ctx.h, _abi.MATTE8, ctypes.c_void_p(src.ctypes.data), 4, _abi.SRGBA8,
                          ctypes.c_void_p(src.ctypes.data), 4, 4, 4, _abi.HOST)
    assert rc == _abi.ERR_ARG
