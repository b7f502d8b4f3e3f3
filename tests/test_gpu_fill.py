"""Fill parity: the CUDA path (through the C ABI) against the oracle, bit-exact.

Known answers from footile's tests (src/fig.rs:691-794), seeded random paths, and
the quirks of the reference: the 65,535-vertex cap (fig.rs:428-442), the shift
of figures whose top row is negative (fig.rs:496-499), the Matte8 overwrite of
every row from the top row down (fig.rs:629-636), wrapping Fixed arithmetic
(fixed.rs:40-56, fig.rs:116-119) and the close-pop of a vertex equal to the
sub-figure start (fig.rs:373-383).
"""
import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, workloads
from footile_gb300._lib import FootileError
from footile_gb300.path import Path2D, PathOp, ops_array
from footile_gb300.plotter import Plotter
from helpers import assert_same, fig_ops, gpu_vs_oracle, new_raster
from test_oracle_golden import FIG_CASES

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["warp", "cta"])
def rasteriser(request, ctx):
    """Small canvases go to the warp rasteriser by default; a tuning with
    warp_max_side 0 sends every path to the CTA rasteriser, so both kernels are
    checked."""
    if request.param == "cta":
        ctx.tune(warp_max_side=0)
    return request.param


@pytest.mark.parametrize("name", sorted(FIG_CASES))
def test_fig_known_answers(ctx, name):
    pts, w, h, want = FIG_CASES[name]
    r = np.zeros((h, w), np.uint8)
    Plotter(r, context=ctx).fill(_abi.NONZERO, fig_ops(pts))
    assert r.ravel().tolist() == want


def test_fig_3x3_rgba8p(ctx):
    r = np.zeros((3, 3, 4), np.uint8)
    Plotter(r, context=ctx).fill(_abi.NONZERO, fig_ops([(1.0, 2.0), (1.0, 3.0), (2.0, 3.0), (2.0, 2.0)]),
                                 (99, 99, 99, 255))
    want = np.zeros((3, 3, 4), np.uint8)
    want[2, 1] = (99, 99, 99, 255)
    assert np.array_equal(r, want)


@pytest.mark.parametrize("seed", range(12))
@pytest.mark.parametrize("rule", [_abi.NONZERO, _abi.EVENODD])
def test_random_paths_matte8(ctx, rasteriser, seed, rule):
    rng = np.random.default_rng(100 + seed)
    w = int(rng.integers(1, 300))
    h = int(rng.integers(1, 300))
    side = max(w, h) * float(rng.uniform(0.5, 1.5))
    ops = workloads.random_path(rng, side, int(rng.integers(1, 60)), n_sub=int(rng.integers(1, 4)),
                                close=bool(rng.integers(0, 2)))
    got, want, st, _, err = gpu_vs_oracle(ctx, ops, w, h, _abi.MATTE8, rule, init=int(rng.integers(0, 256)))
    assert st == 0 and err is None
    assert_same(got, want, f"seed {seed}")


@pytest.mark.parametrize("seed", range(6))
def test_random_paths_rgba8p(ctx, rasteriser, seed):
    rng = np.random.default_rng(200 + seed)
    w, h = int(rng.integers(1, 200)), int(rng.integers(1, 200))
    ops = workloads.random_path(rng, max(w, h), 40, n_sub=2)
    a = int(rng.integers(0, 256))
    clr = tuple(int(v) for v in rng.integers(0, a + 1, 3)) + (a,)
    init = rng.integers(0, 256, (h, w, 4)).astype(np.uint8)
    want = init.copy()
    oracle.fill(seed % 2, ops, want, _abi.RGBA8P, clr)
    got = init.copy()
    Plotter(got, context=ctx).fill(seed % 2, ops, clr)
    assert_same(got, want, f"rgba seed {seed}")


def test_single_path_256(ctx, rasteriser):
    ops, w, h, clr = workloads.single_path_256()
    got, want, st, _, err = gpu_vs_oracle(ctx, ops, w, h)
    assert err is None
    assert_same(got, want, "matte")
    got, want, st, _, err = gpu_vs_oracle(ctx, ops, w, h, _abi.RGBA8P, clr=tuple(clr))
    assert_same(got, want, "rgba")


def test_empty_and_degenerate(ctx, rasteriser):
    for ops in [ops_array([]), ops_array([PathOp.Move(3, 3)]), ops_array([PathOp.Close(), PathOp.Close()]),
                fig_ops([(1, 1), (1, 1), (1, 1)]), fig_ops([(1, 1), (5, 1), (9, 1)]),
                ops_array([PathOp.PenWidth(3.0)])]:
        got, want, st, _, err = gpu_vs_oracle(ctx, ops, 12, 7, init=9)
        assert err is None
        assert_same(got, want, str(ops["kind"].tolist()))


def test_negative_top_row_shift(ctx, rasteriser):
    # fig.rs:496-499: raster row 0 receives scan row top_row when top_row < 0
    ops = fig_ops([(2.5, -5.25), (20.0, 3.0), (6.0, 14.5), (1.0, 9.0)])
    got, want, st, _, err = gpu_vs_oracle(ctx, ops, 24, 16, init=3)
    assert_same(got, want, "negative top row")
    ops = fig_ops([(2.5, -40000.0), (20.0, 3.0), (6.0, 14.5)])  # saturated Fixed y
    got, want, *_ = gpu_vs_oracle(ctx, ops, 24, 16, init=3)
    assert_same(got, want, "saturated top row")


def test_rows_above_top_untouched(ctx):
    ops = fig_ops([(2.0, 10.0), (20.0, 12.0), (6.0, 14.5)])
    got, want, *_ = gpu_vs_oracle(ctx, ops, 24, 16, init=77)
    assert (got[:10] == 77).all()
    assert_same(got, want, "rows above top")


def test_x_out_of_bounds(ctx, rasteriser):
    for pts in [[(-30.0, 0.0), (-20.0, 9.0), (5.5, 4.5)], [(10.0, 0.0), (60.0, 9.0), (45.5, 4.5)],
                [(-1e6, 0.5), (1e6, 7.25), (3.0, 9.0)]]:
        got, want, *_ = gpu_vs_oracle(ctx, fig_ops(pts), 17, 11)
        assert_same(got, want, str(pts))


def test_wrapping_widdershins_long_edges(ctx):
    # |dx*dy| beyond 32768 px^2 wraps the Fixed products of the direction test
    pts = [(0.5, 0.5), (30000.0, 1.5), (29000.0, 3.0), (1.0, 20000.0)]
    got, want, *_ = gpu_vs_oracle(ctx, fig_ops(pts), 64, 48)
    assert_same(got, want, "wrapping direction")


def test_close_pops_start_point(ctx, rasteriser):
    # a sub-figure that returns to its start loses the closing vertex
    pts = [(2.0, 2.0), (12.0, 3.0), (8.0, 11.0), (2.0, 2.0)]
    ops = ops_array([PathOp.Move(*pts[0])] + [PathOp.Line(*p) for p in pts[1:]] + [PathOp.Close()] +
                    [PathOp.Move(5, 5), PathOp.Line(5, 5), PathOp.Close(), PathOp.Line(9, 1), PathOp.Line(13, 9)])
    got, want, *_ = gpu_vs_oracle(ctx, ops, 16, 14)
    assert_same(got, want, "close pop")


def test_nan_points(ctx):
    nan = float("nan")
    ops = ops_array([PathOp.Move(1, 1), PathOp.Line(nan, 5), PathOp.Line(9, nan), PathOp.Line(12, 12)])
    got, want, st, _, err = gpu_vs_oracle(ctx, ops, 16, 16)
    assert st == 0 and err is None
    assert_same(got, want, "nan line")
    ops = ops_array([PathOp.Move(1, 1), PathOp.Quad(nan, 5, 9, 9), PathOp.Line(12, 1)])
    got, want, st, _, err = gpu_vs_oracle(ctx, ops, 16, 16)
    assert st == _abi.ERR_ARG
    assert isinstance(err, FootileError) and err.code == _abi.ERR_ARG
    assert_same(got, want, "nan quad")


@pytest.mark.parametrize("tol", [0.01, 0.3, 2.0])
def test_tolerance_and_transform(ctx, tol):
    rng = np.random.default_rng(7)
    ops = workloads.random_path(rng, 60, 30, n_sub=2)
    xf = (1.5, 0.25, 3.0, -0.5, 1.25, 40.0)
    got, want, *_ = gpu_vs_oracle(ctx, ops, 128, 128, tolerance=tol, transform=xf)
    assert_same(got, want, f"tol {tol}")


def test_pen_width_persists(ctx):
    r = np.zeros((8, 8), np.uint8)
    p = Plotter(r, context=ctx)
    ctx.set_pen_width(1.0)
    p.fill(_abi.NONZERO, Path2D().pen_width(5.5).move_to(1, 1).line_to(6, 2).line_to(3, 6).finish())
    assert p.pen_width() == 5.5
    p.fill(_abi.NONZERO, fig_ops([(1, 1), (6, 2), (3, 6)]))
    assert p.pen_width() == 5.5


def test_vertex_cap_65535(ctx, rasteriser):
    # more than 65,535 vertices: footile keeps the first 65,535 (fig.rs:428-442)
    rng = np.random.default_rng(11)
    n = 70000
    xy = rng.random((n, 2)).astype(np.float32) * np.float32(64)
    ops = np.zeros(n + 1, dtype=_abi.OP_DTYPE)
    ops["kind"][0] = _abi.OP_MOVE
    ops["kind"][1:n] = _abi.OP_LINE
    ops["v"][:n, :2] = xy
    ops["kind"][n] = _abi.OP_CLOSE
    assert len(oracle.fig_points(ops)) == 65535
    got, want, *_ = gpu_vs_oracle(ctx, ops, 64, 64)
    assert_same(got, want, "cap")


def test_vertex_cap_with_closing_pop(ctx):
    # the sub-figure open at the cap returns to its start: the final close pops
    n = 65534
    xy = np.zeros((n + 2, 2), np.float32)
    ang = np.linspace(0, 2 * np.pi, n, endpoint=False)
    xy[:n, 0] = 32 + 30 * np.cos(ang)
    xy[:n, 1] = 32 + 30 * np.sin(ang)
    xy[n] = (40.0, 3.0)
    xy[n + 1] = xy[0]
    ops = np.zeros(n + 2, dtype=_abi.OP_DTYPE)
    ops["kind"][:] = _abi.OP_LINE
    ops["kind"][0] = _abi.OP_MOVE
    ops["v"][:, :2] = xy
    pts = oracle.fig_points(ops)
    got, want, *_ = gpu_vs_oracle(ctx, ops, 64, 64)
    assert_same(got, want, f"cap pop ({len(pts)} vertices)")


def test_scene_4096_capped(ctx):
    # 1,000 sub-paths flatten to millions of vertices; footile keeps 65,535
    ops, w, h, clr = workloads.scene_4096()
    for rule in (_abi.NONZERO, _abi.EVENODD):
        got, want, *_ = gpu_vs_oracle(ctx, ops, w, h, rule=rule)
        assert_same(got, want, f"scene rule {rule}")


def test_warp_overflow_hands_path_to_cta(ctx):
    # a batch large enough for the warp rasteriser, where a few figures have more
    # vertices than a warp holds (9,000): those warps hand their paths to the CTA
    # kernel; nothing may change in the result
    from footile_gb300.plotter import fill_batch, pack_batch
    rng = np.random.default_rng(21)
    paths_ops, sizes = [], []
    for i in range(400):
        if i % 100 == 7:
            n = 9000
            ang = np.sort(rng.random(n)) * 2 * np.pi
            rad = 20 + 10 * rng.random(n)
            ops = np.zeros(n + 1, dtype=_abi.OP_DTYPE)
            ops["kind"][0] = _abi.OP_MOVE
            ops["kind"][1:n] = _abi.OP_LINE
            ops["v"][:n, 0] = 32 + rad * np.cos(ang)
            ops["v"][:n, 1] = 32 + rad * np.sin(ang)
            ops["kind"][n] = _abi.OP_CLOSE
        else:
            ops = workloads.random_path(rng, 64, int(rng.integers(2, 20)))
        paths_ops.append(ops)
        sizes.append(64)
    ops, paths, nbytes = pack_batch(paths_ops, sizes)
    want = np.zeros(nbytes, np.uint8)
    oracle.fill_batch(0, _abi.NONZERO, ops, paths, _abi.MATTE8, want, n_threads=8)
    got = np.zeros(nbytes, np.uint8)
    st = fill_batch(ctx, ops, paths, _abi.MATTE8, got)
    assert (st == 0).all()
    assert_same(got, want, "overflow batch")


@pytest.mark.parametrize("init_kind", ["zero", "random"])
@pytest.mark.parametrize("stroke", [False, True])
def test_scene_4096_rgba8p(ctx, stroke, init_kind):
    """The benchmark's 4096x4096 scene composited onto Rgba8p: the NonZero fill, and the
    stroke at width 8 with round joins, each bit-exact against the oracle; on the
    benchmark's zeroed canvas and on random bytes (where every call's alpha-0 SrcOver
    from its top row down changes the destination)."""
    from footile_gb300.path import PathOp, ops_array
    ops, w, h, clr = workloads.scene_4096()
    init = 0 if init_kind == "zero" else np.random.default_rng(2).integers(0, 256, (h, w, 4)).astype(np.uint8)
    if stroke:
        ops = np.concatenate([ops_array([PathOp.PenWidth(8.0)]), ops])
        got, want, st_o, _, err = gpu_vs_oracle(ctx, ops, w, h, fmt=_abi.RGBA8P, clr=tuple(int(c) for c in clr),
                                                init=init, stroke=True, join=_abi.JOIN_ROUND, miter_limit=0.0)
    else:
        got, want, st_o, _, err = gpu_vs_oracle(ctx, ops, w, h, fmt=_abi.RGBA8P, clr=tuple(int(c) for c in clr),
                                                init=init)
    assert err is None and st_o == 0
    assert_same(got, want, f"scene Rgba8p stroke={stroke} ({init_kind} canvas)")


@pytest.mark.parametrize("stage", [0, 1, 2])
def test_large_rgba8p_compositing_paths(ctx, stage):
    """A single Rgba8p call of at least 1 Mpx is composited from its Matte8 coverage by the
    TMA streaming pass (stage 0, built-in), or by the tile compositor with its tile staged
    by TMA (1) or in place (2); all give the oracle's bytes, on random canvas bytes."""
    ctx.tune(tile_stage=stage)
    rng = np.random.default_rng(50 + stage)
    w, h = 1280, 1000
    ops = workloads.random_path(rng, 1280, 300, n_sub=3)
    init = rng.integers(0, 256, (h, w, 4)).astype(np.uint8)
    got, want, st_o, _, err = gpu_vs_oracle(ctx, ops, w, h, fmt=_abi.RGBA8P, clr=(30, 10, 5, 120), init=init,
                                            rule=_abi.EVENODD)
    assert err is None
    assert_same(got, want, f"stage {stage}")


def test_large_rgba8p_unaligned_rows(ctx):
    """Rows 4,004 bytes apart admit no TMA tensor map: the single large call is composited
    in place by the tile compositor."""
    rng = np.random.default_rng(61)
    w, h = 1001, 1100
    ops = workloads.random_path(rng, 1100, 200, n_sub=2)
    init = rng.integers(0, 256, (h, w, 4)).astype(np.uint8)
    got, want, _, _, err = gpu_vs_oracle(ctx, ops, w, h, fmt=_abi.RGBA8P, clr=(9, 200, 14, 230), init=init)
    assert err is None
    assert_same(got, want, "unaligned rows")
