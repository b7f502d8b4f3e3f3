"""The grid-wide figure build (k_gb_* in footile_gb300/csrc/ft_kernels.cu) against the
oracle: single fills sent to the one-build compositor (split_px 1) with the figure built
by the whole GPU (fig_build 2) and, beside it, by one CTA (fig_build 1).  Random line
paths with coincident points, returns to the start, Moves and Closes in every order;
random curve paths under a transform; the 65,535-vertex cap crossed at many offsets;
status words, the pen width after the call, and un-capped figures."""
import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, workloads
from footile_gb300.path import Path2D, PathOp, ops_array
from footile_gb300.plotter import Plotter

from helpers import assert_same, gpu_vs_oracle
from test_grid_build_model import random_lines

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[2, 1], ids=["grid", "cta"])
def build(request, ctx):
    ctx.tune(split_px=1, fig_build=request.param)
    return request.param


@pytest.mark.parametrize("seed", range(12))
def test_random_line_paths(ctx, build, seed):
    rng = np.random.default_rng(100 + seed)
    ops = random_lines(rng, int(rng.integers(1, 3000)), grid=int(rng.integers(2, 60)))
    ops["v"][:, :2] *= np.float32(4.0)  # grid points 1 px apart on a 64 px canvas
    fmt = _abi.MATTE8 if seed % 2 else _abi.RGBA8P
    rule = _abi.NONZERO if seed % 3 else _abi.EVENODD
    got, want, *_ = gpu_vs_oracle(ctx, ops, 64, 64, fmt=fmt, rule=rule, clr=(200, 40, 90, 180), init=37)
    assert_same(got, want, f"lines seed {seed}")


@pytest.mark.parametrize("seed", range(6))
def test_random_curve_paths(ctx, build, seed):
    rng = np.random.default_rng(200 + seed)
    ops = workloads.random_path(rng, 300, int(rng.integers(20, 400)), n_sub=int(rng.integers(1, 12)),
                                close=bool(seed % 2))
    xf = (1.25, 0.125, 5.0, -0.25, 0.75, 9.0) if seed % 3 == 0 else _abi.IDENTITY
    got, want, *_ = gpu_vs_oracle(ctx, ops, 384, 320, fmt=_abi.RGBA8P, clr=(20, 200, 90, 255), init=3,
                                  tolerance=(0.05, 0.3, 1.0)[seed % 3], transform=xf)
    assert_same(got, want, f"curves seed {seed}")


@pytest.mark.parametrize("extra", [-2, -1, 0, 1, 3])
@pytest.mark.parametrize("tail", ["dup", "back", "move", "close"])
def test_cap_crossing(ctx, build, extra, tail):
    n = _abi.MAX_POINTS + extra
    k = np.arange(n)
    ops = np.zeros(n + 3, dtype=_abi.OP_DTYPE)
    ops["kind"][0] = _abi.OP_MOVE
    ops["kind"][1:n] = _abi.OP_LINE
    ops["v"][:n, 0] = ((k * 7919) % 256).astype(np.float32) * np.float32(0.25)
    ops["v"][:n, 1] = ((k * 104729) % 240).astype(np.float32) * np.float32(0.25)
    x, y = float(ops["v"][n - 1, 0]), float(ops["v"][n - 1, 1])
    x0, y0 = float(ops["v"][0, 0]), float(ops["v"][0, 1])
    t = ops_array({
        "dup": [PathOp.Line(x, y), PathOp.Line(33.0, 21.0)],
        "back": [PathOp.Line(x0, y0), PathOp.Line(x0, y0)],
        "move": [PathOp.Move(5.0, 5.0), PathOp.Line(40.0, 9.0), PathOp.Line(12.0, 50.0)],
        "close": [PathOp.Line(x0, y0), PathOp.Close(), PathOp.Line(30.0, 30.0)],
    }[tail])
    ops[n:n + len(t)] = t
    ops = ops[:n + len(t)]
    got, want, *_ = gpu_vs_oracle(ctx, ops, 64, 60, rule=_abi.EVENODD)
    assert_same(got, want, f"cap {tail} {extra}")


def test_many_short_subfigures_over_the_cap(ctx, build):
    rng = np.random.default_rng(9)
    ops = random_lines(rng, 150000, grid=200, p_move=0.2, p_close=0.2, p_back=0.2)
    ops["v"][:, :2] *= np.float32(1.5)
    got, want, *_ = gpu_vs_oracle(ctx, ops, 80, 80, fmt=_abi.RGBA8P, clr=(9, 99, 199, 255), init=200)
    assert_same(got, want, "short sub-figures")


def test_status_and_pen_width(ctx, build):
    nan = float("nan")
    ops = ops_array([PathOp.PenWidth(3.0), PathOp.Move(1, 1), PathOp.Quad(nan, 5, 9, 9), PathOp.Line(12, 1),
                     PathOp.PenWidth(6.5), PathOp.Close()])
    got, want, st, sw, err = gpu_vs_oracle(ctx, ops, 16, 16)
    assert st == _abi.ERR_ARG and err is not None and err.code == _abi.ERR_ARG
    assert_same(got, want, "nan quad")
    r = np.zeros((8, 8), np.uint8)
    p = Plotter(r, context=ctx)
    ctx.set_pen_width(1.0)
    p.fill(_abi.NONZERO, Path2D().pen_width(5.5).move_to(1, 1).line_to(6, 2).pen_width(2.5).line_to(3, 6)
           .finish())
    assert p.pen_width() == 2.5
    p.fill(_abi.NONZERO, ops_array([PathOp.Move(1, 1), PathOp.Line(6, 2), PathOp.Line(3, 6)]))
    assert p.pen_width() == 2.5


def test_empty_and_vertexless_paths(ctx, build):
    for ops in ([PathOp.Close()], [PathOp.PenWidth(2.0), PathOp.Close(), PathOp.Close()],
                [PathOp.Move(3, 3)], [PathOp.Move(3, 3), PathOp.Line(3, 3), PathOp.Close()]):
        got, want, *_ = gpu_vs_oracle(ctx, ops_array(ops), 8, 8, fmt=_abi.RGBA8P, clr=(1, 2, 3, 4), init=77)
        assert_same(got, want, "empty")


@pytest.mark.parametrize("cap", [80000, 4 << 20])
def test_uncapped(ctx, build, cap):
    ops = workloads.random_path(np.random.default_rng(17), 512, 100, n_sub=120, close=True)
    want = np.zeros((512, 512, 4), np.uint8)
    oracle.fill(_abi.NONZERO, ops, want, _abi.RGBA8P, (30, 120, 200, 255), fig_cap=cap)
    ctx.set_figure_cap(cap)
    try:
        got = np.zeros_like(want)
        Plotter(got, context=ctx).fill(_abi.NONZERO, ops, (30, 120, 200, 255))
    finally:
        ctx.set_figure_cap(0)
    assert_same(got, want, f"un-capped {cap}")


def test_raw_arrays_grow(ctx):
    """A first path sizes the raw vertex arrays; a path with far more raw vertices per op
    (long cubics) makes the build grow them and run again."""
    ctx.tune(split_px=1, fig_build=2)
    small = ops_array([PathOp.Move(1, 1), PathOp.Line(60, 3), PathOp.Line(30, 60)])
    got, want, *_ = gpu_vs_oracle(ctx, small, 64, 64)
    assert_same(got, want, "small")
    ops = [PathOp.Move(0, 0)]
    rng = np.random.default_rng(5)
    for _ in range(200000):
        ops.append(PathOp.Cubic(*(rng.random(6) * 4000).astype(np.float32).tolist()))
    ops = ops_array(ops)
    got, want, *_ = gpu_vs_oracle(ctx, ops, 1000, 900, tolerance=0.05)
    assert_same(got, want, "long cubics")


def probe_boundary_ops(lead, big, n_quads=20000):
    """Lines and quads whose every raw vertex is distinct: after `lead` lines, `big` quads of
    64 leaves, then quads of 32.  The first 2,048 ops (the probe of a long path) hold
    65,474 - 31 * lead + 32 * big raw vertices."""
    ops = [PathOp.Move(0.0, 700.0)]
    ops += [PathOp.Line(0.125 + 0.0625 * k, 700.0 - 0.125 * k) for k in range(lead)]
    x, y = 0.125 + 0.0625 * lead, 700.0
    ops.append(PathOp.Line(x, y))
    for k in range(n_quads):
        h = 1280.0 if k < big else 320.0
        ops.append(PathOp.Quad(x + 0.125, y - h, x + 0.25, y))
        x += 0.25
    return ops


# (lead, big): the probe's raw vertices 65,804 / 65,556 (the cap inside), 65,525 (after it),
# 65,503, 65,535 (its last vertex: the cap just after it) and 65,567
PROBE_CASES = [(10, 20), (18, 20), (19, 20), (29, 29), (29, 30), (29, 31)]


@pytest.mark.parametrize("lead,big", PROBE_CASES)
def test_cap_near_the_probe_boundary(ctx, lead, big):
    """Long paths are built first over their first 2,048 ops; when the cap is reached
    there, the build over all ops is skipped."""
    ctx.tune(split_px=1, fig_build=2)
    ops = ops_array(probe_boundary_ops(lead, big))
    got, want, *_ = gpu_vs_oracle(ctx, ops, 5010, 720, rule=_abi.EVENODD)
    assert_same(got, want, f"lead {lead} big {big}")


# ---- strokes: the stroker's points, sub-strokes and outline built by the whole GPU

def random_stroke_ops(rng, n_ops, side, grid=None):
    """Moves, lines, quads, cubics, closes and pen widths; with `grid`, points on a coarse
    grid so that coincident stroke points and one-point sub-strokes occur."""
    ops = []
    for _ in range(n_ops):
        u = rng.random()
        pt = (lambda: (float(rng.integers(0, grid)) * side / grid, float(rng.integers(0, grid)) * side / grid)) \
            if grid else (lambda: tuple(float(v) for v in rng.random(2) * side))
        if u < 0.1 or not ops:
            ops.append(PathOp.Move(*pt()))
        elif u < 0.18:
            ops.append(PathOp.Close())
        elif u < 0.22:
            ops.append(PathOp.PenWidth(float(rng.uniform(0.5, 9.0))))
        elif u < 0.55:
            ops.append(PathOp.Line(*pt()))
        elif u < 0.8:
            ops.append(PathOp.Quad(*pt(), *pt()))
        else:
            ops.append(PathOp.Cubic(*pt(), *pt(), *pt()))
    return ops_array(ops)


@pytest.mark.parametrize("join", [_abi.JOIN_MITER, _abi.JOIN_BEVEL, _abi.JOIN_ROUND])
@pytest.mark.parametrize("seed", range(4))
def test_random_strokes(ctx, build, join, seed):
    rng = np.random.default_rng(300 + seed)
    ops = random_stroke_ops(rng, int(rng.integers(5, 600)), 200.0, grid=(6 if seed % 2 else None))
    xf = (1.25, 0.125, 5.0, -0.25, 0.75, 9.0) if seed == 2 else _abi.IDENTITY
    fmt = _abi.RGBA8P if seed % 2 else _abi.MATTE8
    got, want, st, sw, err = gpu_vs_oracle(ctx, ops, 256, 230, fmt=fmt, clr=(40, 90, 200, 230), init=11,
                                           stroke=True, join=join, miter_limit=(4.0, 1.5, 10.0, 2.0)[seed],
                                           s_width=(1.0, 3.5, 6.0, 0.75)[seed], transform=xf,
                                           tolerance=(0.3, 0.1, 0.5, 1.0)[seed])
    assert_same(got, want, f"stroke {join} {seed}")
    assert (err.code if err else 0) == st
    assert ctx.pen_width() == sw


@pytest.mark.parametrize("tail", ["close", "move", "line", "closes_after"])
@pytest.mark.parametrize("extra", [-1, 0, 2])
def test_stroke_point_cap(ctx, build, tail, extra):
    """More stroke points than 65,535: points from the cap on are dropped, and the last
    sub-stroke's joined flag comes from the close events after its last kept point."""
    n = _abi.MAX_POINTS + extra
    k = np.arange(n)
    ops = np.zeros(n + 4, dtype=_abi.OP_DTYPE)
    ops["kind"][0] = _abi.OP_MOVE
    ops["kind"][1:n] = _abi.OP_LINE
    ops["v"][:n, 0] = ((k * 7919) % 200).astype(np.float32) * np.float32(0.5) + np.float32(8)
    ops["v"][:n, 1] = ((k * 104729) % 180).astype(np.float32) * np.float32(0.5) + np.float32(8)
    t = ops_array({
        "close": [PathOp.Close(), PathOp.Line(30.0, 30.0)],
        "move": [PathOp.Move(5.0, 5.0), PathOp.Line(40.0, 9.0)],
        "line": [PathOp.Line(3.0, 7.0), PathOp.Line(50.0, 70.0)],
        "closes_after": [PathOp.Line(60.0, 20.0), PathOp.Move(1.0, 1.0), PathOp.Close()],
    }[tail])
    ops[n:n + len(t)] = t
    ops = ops[:n + len(t)]
    got, want, *_ = gpu_vs_oracle(ctx, ops, 116, 106, stroke=True, join=_abi.JOIN_ROUND, s_width=0.8)
    assert_same(got, want, f"stroke cap {tail} {extra}")


def test_stroke_outline_grows_raw_arrays(ctx):
    """A small stroke sizes the arrays; then wide round joins on 70,000 short segments give
    an outline of far more raw vertices than that, and the build grows its arrays and
    runs again."""
    ctx.tune(split_px=1, fig_build=2)
    small = ops_array([PathOp.Move(10, 10), PathOp.Line(60, 13), PathOp.Line(30, 60)])
    got, want, *_ = gpu_vs_oracle(ctx, small, 64, 64, stroke=True)
    assert_same(got, want, "small stroke")
    rng = np.random.default_rng(12)
    ops = [PathOp.PenWidth(60.0), PathOp.Move(100.0, 100.0)]
    for _ in range(70000):
        ops.append(PathOp.Line(*(rng.random(2) * 400 + 50).astype(np.float32).tolist()))
    got, want, *_ = gpu_vs_oracle(ctx, ops_array(ops), 500, 500, stroke=True, join=_abi.JOIN_ROUND,
                                  tolerance=0.05)
    assert_same(got, want, "wide round joins")


@pytest.mark.parametrize("lead,big", PROBE_CASES)
def test_stroke_point_cap_near_the_probe_boundary(ctx, lead, big):
    """Long stroke paths collect their points first over their first 2,048 ops; when the
    65,535-point cap is reached there the points are complete."""
    ctx.tune(split_px=1, fig_build=2)
    ops = probe_boundary_ops(lead, big) + [PathOp.Close()]
    got, want, *_ = gpu_vs_oracle(ctx, ops_array(ops), 5010, 720, stroke=True, join=_abi.JOIN_BEVEL,
                                  s_width=0.5)
    assert_same(got, want, f"stroke lead {lead} big {big}")


@pytest.mark.parametrize("stroke", [False, True])
def test_composite_batch_of_one_offset_path(ctx, stroke):
    """ft_composite_batch of one path whose ops start after 500 ops of another path: the
    grid-wide build reads the path's ops from its op_begin; the canvas starts random."""
    from footile_gb300.plotter import composite_batch
    ctx.tune(fig_build=2)
    rng = np.random.default_rng(31)
    junk = workloads.random_path(rng, 300, 500, n_sub=1)
    path = workloads.random_path(rng, 300, 700, n_sub=9, close=not stroke)
    if stroke:
        path = np.concatenate([ops_array([PathOp.PenWidth(3.5)]), path])
    ops = np.concatenate([junk, path])
    paths = np.zeros(1, dtype=_abi.PATH_DTYPE)
    paths[0]["op_begin"] = len(junk)
    paths[0]["n_ops"] = len(path)
    paths[0]["width"] = 320
    paths[0]["height"] = 300
    paths[0]["clr"] = (90, 30, 160, 200)
    init = rng.integers(0, 256, (300, 320, 4)).astype(np.uint8)
    want = init.copy()
    oracle.composite(int(stroke), _abi.EVENODD, ops, paths, _abi.RGBA8P, want, s_width=1.0)
    got = init.copy()
    ctx.set_pen_width(1.0)
    composite_batch(ctx, ops, paths, _abi.RGBA8P, got, rule=_abi.EVENODD, stroke=stroke)
    assert_same(got, want, f"one offset path, stroke {stroke}")


@pytest.mark.parametrize("stroke,join", [(False, None), (True, _abi.JOIN_MITER), (True, _abi.JOIN_ROUND)])
def test_built_in_route_large_paths(ctx, stroke, join):
    """No tuning: a path of more than FT_GRID_BUILD_OPS ops on a 1024x1024 canvas takes the
    grid-wide build by default (with its probe), against the oracle."""
    rng = np.random.default_rng(41 + int(stroke))
    ops = workloads.random_path(rng, 1024, 300, n_sub=10, close=not stroke)
    assert len(ops) > 2048
    kw = dict(stroke=True, join=join, s_width=2.5) if stroke else dict(rule=_abi.NONZERO)
    got, want, st, sw, err = gpu_vs_oracle(ctx, ops, 1024, 1024, fmt=_abi.RGBA8P, clr=(10, 200, 120, 180),
                                           init=5, **kw)
    assert_same(got, want, f"built-in route, stroke {stroke}")
    assert (err.code if err else 0) == st


def test_stroke_points_grow_raw_arrays(ctx):
    """8,000 long cubics at tolerance 0.01: over a million raw stroke points, more than the
    arrays first hold (64 per op, at least 2^20); the build grows them and runs again."""
    ctx.tune(split_px=1, fig_build=2)
    rng = np.random.default_rng(19)
    ops = [PathOp.Move(10.0, 10.0)]
    for _ in range(8000):
        ops.append(PathOp.Cubic(*(rng.random(6) * 990 + 5).astype(np.float32).tolist()))
    got, want, *_ = gpu_vs_oracle(ctx, ops_array(ops), 1000, 1000, stroke=True, join=_abi.JOIN_MITER,
                                  tolerance=0.01, s_width=1.5)
    assert_same(got, want, "many stroke points")
