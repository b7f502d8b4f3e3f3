"""Un-capped figures on the GPU (`ft_set_figure_cap`) against the oracle's un-capped Fig
(u32 vertex ids, footile's algorithm otherwise): bit-exact masks and composites for
figures of 80 k to 1.2 M vertices, a cap between footile's and the figure's size, and
footile's cap restored by 0."""
import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, workloads
from footile_gb300._lib import FootileError
from footile_gb300.plotter import Plotter, composite_batch, pack_batch

from test_uncapped_oracle import squares

pytestmark = pytest.mark.gpu


def scene(n_sub, segs, side, seed):
    return workloads.random_path(np.random.default_rng(seed), side, segs, n_sub=n_sub, close=True)


@pytest.mark.parametrize("rule", [_abi.NONZERO, _abi.EVENODD])
def test_disjoint_squares_all_kept(ctx, rule):
    ops, _ = squares(10, 30, 226, jitter_seed=3)  # 90,400 vertices
    want = np.zeros((300, 300), np.uint8)
    oracle.fill(rule, ops, want, _abi.MATTE8, fig_cap=1 << 20)
    capped = np.zeros_like(want)
    oracle.fill(rule, ops, capped, _abi.MATTE8)
    assert not np.array_equal(want, capped)
    ctx.set_figure_cap(1 << 20)
    try:
        assert ctx.figure_cap() == 1 << 20
        got = np.zeros_like(want)
        Plotter(got, context=ctx).fill(rule, ops)
        assert np.array_equal(got, want)
    finally:
        ctx.set_figure_cap(0)
    assert ctx.figure_cap() == _abi.MAX_POINTS


@pytest.mark.parametrize("fmt", [_abi.MATTE8, _abi.RGBA8P])
def test_large_scene(ctx, fmt):
    ops = scene(200, 100, 1024, seed=17)  # ~1.2 M flattened vertices before the cap
    shape = (1024, 1024) if fmt == _abi.MATTE8 else (1024, 1024, 4)
    clr = (30, 120, 200, 255)
    want = np.zeros(shape, np.uint8)
    oracle.fill(_abi.NONZERO, ops, want, fmt, clr, fig_cap=4 << 20)
    capped = np.zeros(shape, np.uint8)
    oracle.fill(_abi.NONZERO, ops, capped, fmt, clr)
    assert not np.array_equal(want, capped)
    ctx.set_figure_cap(4 << 20)
    try:
        got = np.zeros(shape, np.uint8)
        Plotter(got, context=ctx).fill(_abi.NONZERO, ops, clr)
        assert np.array_equal(got, want)
    finally:
        ctx.set_figure_cap(0)


def test_cap_between_and_footile_cap_restored(ctx):
    ops, _ = squares(10, 30, 226, jitter_seed=4)
    mid = np.zeros((300, 300), np.uint8)
    oracle.fill(_abi.NONZERO, ops, mid, _abi.MATTE8, fig_cap=80000)
    ctx.set_figure_cap(80000)
    got = np.zeros_like(mid)
    Plotter(got, context=ctx).fill(_abi.NONZERO, ops)
    assert np.array_equal(got, mid)
    ctx.set_figure_cap(0)
    foot = np.zeros_like(mid)
    oracle.fill(_abi.NONZERO, ops, foot, _abi.MATTE8)
    got0 = np.zeros_like(mid)
    Plotter(got0, context=ctx).fill(_abi.NONZERO, ops)
    assert np.array_equal(got0, foot)
    with pytest.raises(FootileError):
        ctx.set_figure_cap((1 << 26) + 1)


def test_composite_of_uncapped_fills(ctx):
    a, _ = squares(10, 30, 226, jitter_seed=5)
    b = scene(20, 60, 300, seed=9)
    clrs = [[200, 40, 40, 255], [20, 90, 100, 160]]
    ops, paths, _ = pack_batch([a, b], [(300, 300)] * 2, _abi.RGBA8P, clrs)
    init = np.random.default_rng(2).integers(0, 256, (300, 300, 4)).astype(np.uint8)
    want = init.copy()
    for o, c in zip((a, b), clrs):
        oracle.fill(_abi.EVENODD, o, want, _abi.RGBA8P, tuple(c), fig_cap=1 << 20)
    ctx.set_figure_cap(1 << 20)
    try:
        got = init.copy()
        st = composite_batch(ctx, ops, paths, _abi.RGBA8P, got, rule=_abi.EVENODD)
        assert (st == 0).all()
        assert np.array_equal(got, want)
    finally:
        ctx.set_figure_cap(0)
