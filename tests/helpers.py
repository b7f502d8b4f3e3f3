"""Shared helpers of the test suite: run the oracle and the CUDA path on the same
inputs and report the first difference."""
import numpy as np

import oracle
from footile_gb300 import _abi
from footile_gb300.path import PathOp, ops_array


def fig_ops(points):
    return ops_array([PathOp.Move(*points[0])] + [PathOp.Line(*p) for p in points[1:]])


def new_raster(w, h, fmt, fill=0):
    if isinstance(fill, np.ndarray):
        return fill.copy()
    if fmt == _abi.MATTE8:
        return np.full((h, w), fill, np.uint8)
    return np.full((h, w, 4), fill, np.uint8)


def first_diff(a, b):
    d = np.argwhere(a != b)
    if len(d) == 0:
        return None
    i = tuple(d[0])
    return f"first diff at {i}: got {a[i]} want {b[i]} ({len(d)} differing values)"


def assert_same(got, want, what=""):
    msg = first_diff(got, want)
    assert msg is None, f"{what}: {msg}"


def gpu_vs_oracle(ctx, ops, w, h, fmt=_abi.MATTE8, rule=_abi.NONZERO, clr=(0, 0, 0, 0), init=0, stroke=False,
                  tolerance=0.3, transform=_abi.IDENTITY, join=_abi.JOIN_MITER, miter_limit=4.0, s_width=1.0):
    """Draw `ops` with the oracle and with the GPU (host-mode C ABI call).  `init` is
    the initial byte of every raster byte, or a whole initial raster (copied)."""
    from footile_gb300.plotter import Plotter
    want = new_raster(w, h, fmt, init)
    params = dict(tolerance=tolerance, transform=transform, join=join, miter_limit=miter_limit)
    if stroke:
        st_o, sw_o = oracle.stroke(ops, want, fmt, clr, s_width=s_width, **params)
    else:
        st_o, sw_o = oracle.fill(rule, ops, want, fmt, clr, s_width=s_width, **params)
    got = new_raster(w, h, fmt, init)
    ctx.set_tolerance(tolerance)
    ctx.set_transform(transform)
    ctx.set_join(join, miter_limit)
    ctx.set_pen_width(s_width)
    p = Plotter(got, context=ctx)
    err = None
    try:
        if stroke:
            p.stroke(ops, clr)
        else:
            p.fill(rule, ops, clr)
    except Exception as e:  # status errors still leave a raster to compare
        err = e
    return got, want, st_o, sw_o, err
