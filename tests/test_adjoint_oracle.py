"""CPU checks of the FP64 gradient oracle of the coverage adjoint.

The oracle defines the differentiable coverage (exact area of the flattened polygon
per pixel, NonZero / EvenOdd) and its gradient with respect to the op floats.  Here
it is checked against itself by central differences with the subdivision tree held
(vertices as Bernstein points of the perturbed floats), against supersampling, and
against footile's integer masks (which approximate the same area)."""

import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, workloads
from footile_gb300.path import Path2D

SHAPE = (Path2D().absolute().move_to(20.3, 10.1).line_to(100.7, 30.2).cubic_to(120, 80, 40, 120, 30.5, 90.25)
         .quad_to(5, 60, 15.5, 40.5).close().finish())
# two sub-figures, one crossing the left and bottom raster edges, and an open one
MULTI = (Path2D().absolute().move_to(-10.5, 20.25).cubic_to(30, -5, 60, 70, 20.5, 60.75).line_to(-4, 50).close()
         .move_to(40.2, 40.7).quad_to(90, 10, 70.3, 75.1).line_to(55.6, 70.2).cubic_to(50, 60, 45, 90, 30.1, 70.4)
         .close().move_to(10, 5).line_to(60.5, 12.25).line_to(30.75, 20.5).finish())


def values(ops):
    return np.array([o["v"] for o in ops], dtype=np.float64)


def test_bernstein_and_float_polygons_agree():
    # the f32 De Casteljau vertices and the f64 Bernstein points of the same tree
    base = values(SHAPE)
    c32, _, _ = oracle.adj_forward(_abi.NONZERO, SHAPE, 128, 128)
    c64, _, _ = oracle.adj_forward(_abi.NONZERO, SHAPE, 128, 128, val=base)
    assert np.abs(c32 - c64).max() < 1e-4


def fd_grad(rule, ops, w, h, target, h_step, transform=_abi.IDENTITY, entries=None):
    base = values(ops)
    fd = np.zeros_like(base)
    idx = entries if entries is not None else [(i, k) for i in range(len(ops)) for k in range(6)]
    for i, k in idx:
        vp, vm = base.copy(), base.copy()
        vp[i, k] += h_step
        vm[i, k] -= h_step
        lp = ((oracle.adj_forward(rule, ops, w, h, val=vp, transform=transform)[0] - target) ** 2).sum()
        lm = ((oracle.adj_forward(rule, ops, w, h, val=vm, transform=transform)[0] - target) ** 2).sum()
        fd[i, k] = (lp - lm) / (2 * h_step)
    return fd


@pytest.mark.parametrize("rule", [_abi.NONZERO, _abi.EVENODD])
@pytest.mark.parametrize("shape", ["shape", "multi"])
def test_oracle_gradient_matches_central_differences(rule, shape):
    ops = SHAPE if shape == "shape" else MULTI
    w = h = 96 if shape == "multi" else 128
    target = np.random.default_rng(5).random((h, w))
    base = values(ops)
    cov, area, st = oracle.adj_forward(rule, ops, w, h, val=base)
    assert st == 0
    g = oracle.adj_backward(rule, ops, w, h, area, 2 * (cov - target), val=base)
    # central differences converge to the analytic gradient as the step shrinks
    fd = fd_grad(rule, ops, w, h, target, 1e-5)
    scale = np.abs(g).max()
    assert scale > 0
    assert np.abs(g - fd).max() / scale < 2e-4
    # Close and the unused slots of Move/Line/Quad take no gradient
    for i, o in enumerate(ops):
        used = {_abi.OP_MOVE: 2, _abi.OP_LINE: 2, _abi.OP_QUAD: 4, _abi.OP_CUBIC: 6}.get(int(o["kind"]), 0)
        assert not g[i, used:].any()


def test_oracle_gradient_at_the_specified_step():
    # h = 1e-2 px: the loss is piecewise quadratic with kinks (|S| = 0 or 1), so central
    # differences at this step agree to about 1 %
    target = np.random.default_rng(5).random((128, 128))
    base = values(SHAPE)
    cov, area, _ = oracle.adj_forward(_abi.NONZERO, SHAPE, 128, 128, val=base)
    g = oracle.adj_backward(_abi.NONZERO, SHAPE, 128, 128, area, 2 * (cov - target), val=base)
    fd = fd_grad(_abi.NONZERO, SHAPE, 128, 128, target, 1e-2)
    assert np.abs(g - fd).max() / np.abs(fd).max() < 3e-2


def test_oracle_gradient_through_transform():
    m = (0.9, 0.2, 5.0, -0.15, 1.1, -3.0)
    target = np.random.default_rng(6).random((128, 128))
    base = values(SHAPE)
    cov, area, _ = oracle.adj_forward(_abi.NONZERO, SHAPE, 128, 128, val=base, transform=m)
    g = oracle.adj_backward(_abi.NONZERO, SHAPE, 128, 128, area, 2 * (cov - target), val=base, transform=m)
    fd = fd_grad(_abi.NONZERO, SHAPE, 128, 128, target, 1e-5, transform=m)
    assert np.abs(g - fd).max() / np.abs(g).max() < 2e-4


def test_oracle_coverage_is_the_polygon_area():
    # 16 x 16 supersampling of the same flattened polygon (footile's Fixed vertices)
    w = h = 128
    cov, _, _ = oracle.adj_forward(_abi.NONZERO, SHAPE, w, h)
    pts = oracle.fig_points(SHAPE).astype(np.float64) / 65536
    s = 16
    ys = (np.arange(h * s) + 0.5) / s
    xs = (np.arange(w * s) + 0.5) / s
    X, Y = np.meshgrid(xs, ys)
    wn = np.zeros_like(X)
    for i in range(len(pts)):
        (x0, y0), (x1, y1) = pts[i], pts[(i + 1) % len(pts)]
        if y0 == y1:
            continue
        xi = x0 + (Y - y0) * (x1 - x0) / (y1 - y0)
        wn += ((y0 <= Y) & (Y < y1) & (X < xi)).astype(float) - ((y1 <= Y) & (Y < y0) & (X < xi)).astype(float)
    ss = np.minimum(np.abs(wn), 1).reshape(h, s, w, s).mean(axis=(1, 3))
    assert np.abs(cov - ss).max() < 4 / 255


def test_oracle_coverage_tracks_footile_masks():
    # footile's 16.16 cell walk approximates the same coverage: close on average
    ops, paths, cov_bytes, _ = workloads.cubics_1024_coverage(n_paths=8)
    for p in paths:
        o = ops[p["op_begin"]:p["op_begin"] + p["n_ops"]]
        cov, _, st = oracle.adj_forward(_abi.NONZERO, o, 128, 128)
        m = np.zeros((128, 128), np.uint8)
        oracle.fill(_abi.NONZERO, o, m, _abi.MATTE8, clr=(255, 255, 255, 255))
        d = np.abs(cov * 255 - m)
        assert st == 0 and d.mean() < 1.5 and np.median(d) < 1.0


def test_oracle_vertex_cap_status():
    n = 70000
    ops = np.zeros(n + 2, dtype=_abi.OP_DTYPE)
    ops["kind"][0] = _abi.OP_MOVE
    ops["kind"][1:-1] = _abi.OP_LINE
    ops["v"][:-1, :2] = np.random.default_rng(1).random((n + 1, 2)) * 50
    ops["kind"][-1] = _abi.OP_CLOSE
    cov, _, st = oracle.adj_forward(_abi.NONZERO, ops, 64, 64)
    assert st == _abi.ERR_CAP and not cov.any()


# ----------------------------------------------------------------------- strokes
STROKE = (Path2D().absolute().pen_width(6.0).move_to(20.3, 30.1).cubic_to(60, 5, 90, 90, 110.2, 40.7)
          .line_to(70.5, 100.25).quad_to(40, 120, 25.5, 80.5).finish())
JOINS = [(_abi.JOIN_MITER, 4.0), (_abi.JOIN_BEVEL, 0.0), (_abi.JOIN_ROUND, 0.0), (_abi.JOIN_MITER, 1.5)]


def test_stroke_outline_nodes_match_the_stroker():
    # the f32 node pass of the stroke adjoint emits exactly the outline footile's
    # stroker emits (the integer oracle's Stroke::path_ops)
    from footile_gb300.path import PathOp, ops_array
    rng = np.random.default_rng(7)
    for i in range(200):
        side = int(rng.integers(16, 200))
        o = workloads.random_path(rng, side, int(rng.integers(1, 25)), n_sub=int(rng.integers(1, 3)),
                                  close=bool(i % 2))
        o = np.concatenate([ops_array([PathOp.PenWidth(float(rng.uniform(0.5, 12)))]), o])
        join = JOINS[i % 4]
        tol = [0.1, 0.3, 1.0][i % 3]
        a = oracle.stroke_outline(o, s_width=1.0, join=join[0], miter_limit=join[1], tolerance=tol)
        b = oracle.adj_stroke_outline(o, s_width=1.0, join=join[0], miter_limit=join[1], tolerance=tol)
        assert len(a) == len(b) and (a["kind"] == b["kind"]).all(), i
        assert np.array_equal(a["v"].view(np.uint32), b["v"].view(np.uint32)), i


@pytest.mark.parametrize("join", JOINS[:3])
def test_stroke_gradient_matches_central_differences(join):
    w = h = 128
    target = np.random.default_rng(5).random((h, w))
    base = values(STROKE)
    kw = dict(join=join[0], miter_limit=join[1])
    cov, area, st = oracle.adj_stroke_forward(STROKE, w, h, val=base, **kw)
    assert st == 0
    g, gsw = oracle.adj_stroke_backward(STROKE, w, h, area, 2 * (cov - target), val=base, **kw)

    def loss(val, sw0=1.0):
        return ((oracle.adj_stroke_forward(STROKE, w, h, val=val, s_width=sw0, **kw)[0] - target) ** 2).sum()
    fd = np.zeros_like(base)
    step = 1e-5
    for i in range(len(STROKE)):
        for k in range(6):
            vp, vm = base.copy(), base.copy()
            vp[i, k] += step
            vm[i, k] -= step
            fd[i, k] = (loss(vp) - loss(vm)) / (2 * step)
    assert np.abs(g - fd).max() / np.abs(fd).max() < 2e-4
    assert g[0, 0] != 0.0  # the PenWidth op receives the width gradient
    # the starting pen width matters only when no PenWidth op precedes the points
    o2 = STROKE[1:]
    b2 = values(o2)
    c2, a2, _ = oracle.adj_stroke_forward(o2, w, h, val=b2, s_width=5.0, **kw)
    _, gsw2 = oracle.adj_stroke_backward(o2, w, h, a2, 2 * (c2 - target), val=b2, s_width=5.0, **kw)
    l = lambda s: ((oracle.adj_stroke_forward(o2, w, h, val=b2, s_width=s, **kw)[0] - target) ** 2).sum()
    fd_sw = (l(5.0 + 1e-5) - l(5.0 - 1e-5)) / 2e-5
    assert abs(gsw2 - fd_sw) <= 2e-4 * max(abs(fd_sw), 1.0)


def test_stroke_coverage_tracks_footile_masks():
    for join in JOINS[:3]:
        cov, _, _ = oracle.adj_stroke_forward(STROKE, 128, 128, join=join[0], miter_limit=join[1])
        m = np.zeros((128, 128), np.uint8)
        oracle.stroke(STROKE, m, _abi.MATTE8, clr=(255,) * 4, join=join[0], miter_limit=join[1])
        assert np.abs(cov * 255 - m).mean() < 1.5


def test_stroke_composite_gradient_matches_central_differences():
    # the FP64 chain: strokes SrcOver'd in order, L2 loss against an RGBA target
    from footile_gb300.adjoint import pack_coverage
    paths_ops, widths, clrs, side = workloads.strokes_16384(n_paths=4, side=48, min_seg=2, max_seg=4)
    ops, paths, _ = pack_coverage(paths_ops, [side] * 4)
    clr = clrs.astype(np.float64) / 255.0
    target = np.random.default_rng(8).random((side * side, 4))
    base = values(ops)
    loss, C, g, gw = oracle.adj_stroke_composite(ops, paths, clr, side, side, target, val=base)
    step = 1e-5
    rng = np.random.default_rng(2)
    entries = [(i, k) for i in range(len(ops)) for k in range(6) if g[i, k] != 0.0]
    for i, k in [entries[j] for j in rng.choice(len(entries), 12, replace=False)]:
        vp, vm = base.copy(), base.copy()
        vp[i, k] += step
        vm[i, k] -= step
        fd = (oracle.adj_stroke_composite(ops, paths, clr, side, side, target, val=vp, grads=False) -
              oracle.adj_stroke_composite(ops, paths, clr, side, side, target, val=vm, grads=False)) / (2 * step)
        assert abs(g[i, k] - fd) <= 2e-4 * np.abs(g).max(), (i, k, g[i, k], fd)


def test_stroke_composite_initial_canvas_gradient():
    # C_0 enters the chain linearly: its gradient matches central differences exactly
    from footile_gb300.adjoint import pack_coverage
    paths_ops, widths, clrs, side = workloads.strokes_16384(n_paths=3, side=32, min_seg=2, max_seg=3)
    ops, paths, _ = pack_coverage(paths_ops, [side] * 3)
    clr = clrs.astype(np.float64) / 255.0
    rng = np.random.default_rng(12)
    target = rng.random((side * side, 4))
    init = rng.random((side * side, 4)) * 0.5
    loss, C, g, gw, g0 = oracle.adj_stroke_composite(ops, paths, clr, side, side, target, init=init)
    _, C_zero, g_zero, _ = oracle.adj_stroke_composite(ops, paths, clr, side, side, target)
    assert not np.allclose(C, C_zero)
    step = 1e-4
    for px, ch in [(int(p), int(q)) for p, q in zip(rng.integers(0, side * side, 10), rng.integers(0, 4, 10))]:
        ip, im = init.copy(), init.copy()
        ip[px, ch] += step
        im[px, ch] -= step
        fd = (oracle.adj_stroke_composite(ops, paths, clr, side, side, target, grads=False, init=ip) -
              oracle.adj_stroke_composite(ops, paths, clr, side, side, target, grads=False, init=im)) / (2 * step)
        assert abs(g0[px, ch] - fd) <= 1e-6 * max(1.0, abs(fd)), (px, ch, g0[px, ch], fd)
