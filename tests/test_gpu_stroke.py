"""Stroke parity: Plotter::stroke on the GPU against the oracle, bit-exact.

Shapes from footile's examples (examples/stroke.rs, stroke2.rs, round.rs, teeth.rs,
drop.rs, fishy.rs), every join style (stroker.rs:13-20, 323-396), open and closed
sub-paths including the Close+Move un-join (stroker.rs:230-236), pen-width changes
(plotter.rs:151-153) and the 65,535-point cap of the stroke (stroker.rs:204-216).
"""
import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, workloads
from footile_gb300.path import Path2D, PathOp, ops_array
from footile_gb300.plotter import fill_batch, pack_batch
from helpers import assert_same, gpu_vs_oracle

pytestmark = pytest.mark.gpu

JOINS = [(_abi.JOIN_MITER, 4.0), (_abi.JOIN_BEVEL, 0.0), (_abi.JOIN_ROUND, 0.0), (_abi.JOIN_MITER, 1.5)]


def example_paths():
    stroke = Path2D().relative().pen_width(5.0).move_to(16.0, 48.0).line_to(32.0, 0.0).line_to(-16.0, -32.0) \
        .close().finish()
    stroke2 = (Path2D().relative().pen_width(6.0).move_to(16.0, 15.0).line_to(32.0, 1.0).line_to(-32.0, 1.0)
               .line_to(32.0, 15.0).line_to(-32.0, 15.0).line_to(32.0, 1.0).line_to(-32.0, 1.0).finish())
    rnd = Path2D().relative().pen_width(40.0).move_to(10.0, 60.0).line_to(50.0, 0.0).line_to(0.0, -50.0).finish()
    teeth = Path2D().relative().move_to(0.0, 8.0)
    for _ in range(4):
        teeth = teeth.line_to(8.0, 8.0).line_to(8.0, -8.0)
    teeth = teeth.move_to(-64.0, 32.0)
    for _ in range(4):
        teeth = teeth.line_to(8.0, 8.0).line_to(8.0, -8.0)
    drop = (Path2D().relative().pen_width(3.0).move_to(50.0, 34.0).cubic_to(4.0, 16.0, 16.0, 28.0, 0.0, 32.0)
            .cubic_to(-16.0, -4.0, -4.0, -16.0, 0.0, -32.0).close().finish())
    fish = (Path2D().relative().pen_width(3.0).move_to(112.0, 24.0).line_to(-32.0, 24.0)
            .cubic_to(-96.0, -48.0, -96.0, 80.0, 0.0, 32.0).line_to(32.0, 24.0).line_to(-16.0, -40.0)
            .close().finish())
    eye = (Path2D().relative().pen_width(2.0).move_to(24.0, 48.0).line_to(8.0, 8.0).move_to(0.0, -8.0)
           .line_to(-8.0, 8.0).finish())
    return {"stroke": (stroke, 64), "stroke2": (stroke2, 64), "round": (rnd, 100), "teeth": (teeth.finish(), 64),
            "drop": (drop, 100), "fish": (fish, 128), "eye": (eye, 128)}


@pytest.mark.parametrize("name", sorted(example_paths()))
@pytest.mark.parametrize("join", JOINS)
def test_example_strokes(ctx, name, join):
    ops, side = example_paths()[name]
    got, want, st, _, err = gpu_vs_oracle(ctx, ops, side, side, stroke=True, join=join[0], miter_limit=join[1])
    assert st == 0 and err is None
    assert_same(got, want, f"{name} {join}")


@pytest.mark.parametrize("seed", range(8))
def test_random_strokes(ctx, seed):
    rng = np.random.default_rng(300 + seed)
    w, h = int(rng.integers(8, 300)), int(rng.integers(8, 300))
    n_sub = int(rng.integers(1, 4))
    ops = workloads.random_path(rng, max(w, h), int(rng.integers(1, 30)), n_sub=n_sub,
                                close=bool(seed % 2))
    pw = ops_array([PathOp.PenWidth(float(rng.uniform(0.5, 14.0)))])
    ops = np.concatenate([pw, ops])
    join = JOINS[seed % len(JOINS)]
    fmt = _abi.MATTE8 if seed < 5 else _abi.RGBA8P
    a = int(rng.integers(1, 256))
    clr = tuple(int(v) for v in rng.integers(0, a + 1, 3)) + (a,)
    got, want, st, sw, err = gpu_vs_oracle(ctx, ops, w, h, fmt, clr=clr, stroke=True, join=join[0],
                                           miter_limit=join[1], tolerance=float(rng.choice([0.1, 0.3, 1.0])))
    assert err is None, err
    assert_same(got, want, f"seed {seed}")
    assert ctx.pen_width() == sw


def test_pen_width_chain_on_device(ctx):
    """Consecutive strokes on device buffers hand the pen width from call to call on the
    device (plotter.rs:151-153), with no host read in between; one call on a 1024² canvas
    takes the large-canvas route (the figure built once, bands composited)."""
    import ctypes
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(17)
    calls = []
    for k in range(6):
        side = 1024 if k == 2 else 96
        ops = workloads.random_path(rng, 96, int(rng.integers(2, 12)), n_sub=1, close=bool(k % 2))
        if k in (0, 3, 4):
            ops = np.concatenate([ops_array([PathOp.PenWidth(float(2 + 2.5 * k))]), ops])
        calls.append((ops, side))
    ctx.set_tolerance(0.3)
    ctx.set_transform(_abi.IDENTITY)
    ctx.set_join(_abi.JOIN_ROUND, 0.0)
    ctx.set_pen_width(1.5)
    clr = (ctypes.c_uint8 * 4)(0, 0, 0, 255)
    keep = []
    for ops, side in calls:
        ops_d = torch.from_numpy(ops.view(np.uint8)).cuda()
        r_d = torch.zeros((side, side), dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        ctx.check(ctx.L.ft_stroke(ctx.h, ctypes.c_void_p(ops_d.data_ptr()), len(ops), _abi.MATTE8, clr,
                                  ctypes.c_void_p(r_d.data_ptr()), side, side, side, _abi.DEVICE))
        keep.append((ops_d, r_d))
    torch.cuda.synchronize()
    sw = 1.5
    for k, ((ops, side), (_, r_d)) in enumerate(zip(calls, keep)):
        want = np.zeros((side, side), np.uint8)
        st, sw = oracle.stroke(ops, want, _abi.MATTE8, (0, 0, 0, 255), s_width=sw, tolerance=0.3,
                               transform=_abi.IDENTITY, join=_abi.JOIN_ROUND, miter_limit=0.0)
        assert st == 0
        assert_same(r_d.cpu().numpy(), want, f"call {k} (pen width {sw})")
    assert ctx.pen_width() == sw


def test_close_then_move_unjoins(ctx):
    # stroker.rs:230-236 — Close then Move leaves the first sub-stroke open
    ops = (Path2D().absolute().pen_width(4.0).move_to(10, 10).line_to(50, 12).line_to(30, 40).close()
           .move_to(60, 60).line_to(90, 62).line_to(70, 90).close().finish())
    got, want, *_ = gpu_vs_oracle(ctx, ops, 100, 100, stroke=True)
    assert_same(got, want, "close+move")
    # Close followed by a line (no Move) keeps it joined
    ops2 = (Path2D().absolute().pen_width(4.0).move_to(10, 10).line_to(50, 12).line_to(30, 40).close()
            .line_to(60, 60).line_to(90, 62).finish())
    got, want, *_ = gpu_vs_oracle(ctx, ops2, 100, 100, stroke=True)
    assert_same(got, want, "close+line")


def test_degenerate_strokes(ctx):
    cases = [ops_array([]), ops_array([PathOp.Move(5, 5)]), ops_array([PathOp.Move(5, 5), PathOp.Close()]),
             ops_array([PathOp.Move(5, 5), PathOp.Line(5, 5), PathOp.Close()]),
             ops_array([PathOp.Move(5, 5), PathOp.Line(20, 5), PathOp.Line(5, 5), PathOp.Close()]),
             ops_array([PathOp.PenWidth(6.0), PathOp.Move(2, 2), PathOp.Line(2, 30), PathOp.Line(2, 40)])]
    for ops in cases:
        for join in JOINS[:3]:
            got, want, st, _, err = gpu_vs_oracle(ctx, ops, 48, 48, stroke=True, join=join[0], miter_limit=join[1])
            assert_same(got, want, f"{ops['kind'].tolist()} {join}")


def test_stroke_point_cap(ctx):
    # 70,000 stroke points: footile keeps 65,535 (stroker.rs:204-216); the outline
    # is then capped again by the figure
    rng = np.random.default_rng(5)
    n = 70000
    ops = np.zeros(n + 2, dtype=_abi.OP_DTYPE)
    ops["kind"][0] = _abi.OP_PEN_WIDTH
    ops["v"][0, 0] = 2.0
    ops["kind"][1] = _abi.OP_MOVE
    ops["kind"][2:] = _abi.OP_LINE
    ops["v"][1:, :2] = rng.random((n + 1, 2)).astype(np.float32) * 120
    ops["kind"][-1] = _abi.OP_CLOSE
    got, want, *_ = gpu_vs_oracle(ctx, ops, 128, 128, stroke=True, join=_abi.JOIN_BEVEL)
    assert_same(got, want, "stroke cap")


def test_scene_4096_stroke_round(ctx):
    # 1,000 sub-paths stroked at width 8 with round joins (butt ends, as footile has no caps)
    ops, w, h, clr = workloads.scene_4096()
    pw = ops_array([PathOp.PenWidth(8.0)])
    ops = np.concatenate([pw, ops])
    got, want, *_ = gpu_vs_oracle(ctx, ops, w, h, _abi.MATTE8, stroke=True, join=_abi.JOIN_ROUND)
    assert_same(got, want, "scene stroke")


def test_stroke_batch(ctx):
    rng = np.random.default_rng(17)
    paths_ops, sizes = [], []
    for i in range(200):
        side = int(rng.integers(16, 200))
        o = workloads.random_path(rng, side, int(rng.integers(2, 25)), close=bool(i % 2))
        paths_ops.append(np.concatenate([ops_array([PathOp.PenWidth(float(rng.uniform(1, 10)))]), o]))
        sizes.append(side)
    ops, paths, nbytes = pack_batch(paths_ops, sizes)
    want = np.zeros(nbytes, np.uint8)
    oracle.fill_batch(1, _abi.NONZERO, ops, paths, _abi.MATTE8, want, n_threads=8)
    got = np.zeros(nbytes, np.uint8)
    st = fill_batch(ctx, ops, paths, _abi.MATTE8, got, stroke=True)
    assert (st == 0).all()
    assert_same(got, want, "stroke batch")
