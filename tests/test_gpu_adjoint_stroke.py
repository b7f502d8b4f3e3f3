"""Stroke coverage adjoint on the GPU (`ft_adjoint_forward` with stroke = 1) against
the FP64 oracle: coverage within 1e-4, gradients of the op floats, PenWidth ops and
starting pen widths within 2e-4 of the oracle's largest entry.  Both cover footile's
f32 outline of each stroke."""
import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, workloads
from footile_gb300.adjoint import Adjoint, pack_coverage
from footile_gb300.path import Path2D, PathOp, ops_array

pytestmark = pytest.mark.gpu

COV_TOL = 1e-4
GRAD_TOL = 2e-4
JOINS = [(_abi.JOIN_MITER, 4.0), (_abi.JOIN_BEVEL, 0.0), (_abi.JOIN_ROUND, 0.0), (_abi.JOIN_MITER, 1.5)]


def strokes(seed, n):
    rng = np.random.default_rng(seed)
    per, sizes, sw = [], [], []
    for i in range(n):
        side = int(rng.integers(24, 160))
        o = workloads.random_path(rng, side, int(rng.integers(1, 20)), n_sub=int(rng.integers(1, 3)),
                                  close=bool(i % 2))
        if i % 3:
            o = np.concatenate([ops_array([PathOp.PenWidth(float(rng.uniform(1.0, 12.0)))]), o])
        per.append(o)
        sizes.append(side)
        sw.append(float(rng.uniform(1.0, 6.0)))
    ops, paths, cov_bytes = pack_coverage(per, sizes)
    paths["s_width"] = sw
    return ops, paths, cov_bytes


def check(ctx, ops, paths, cov_bytes, join, seed=5, transform=_abi.IDENTITY, tolerance=0.3):
    ctx.set_join(*join)
    target = np.random.default_rng(seed).random(cov_bytes // 4)
    adj = Adjoint(ctx)
    cov = np.zeros(cov_bytes // 4, np.float32)
    adj.forward(_abi.NONZERO, ops, paths, cov, stroke=True)
    g_cov = (2.0 * (cov.astype(np.float64) - target)).astype(np.float32)
    g_ops = np.zeros((len(ops), 6), np.float32)
    g_w = np.zeros(len(paths), np.float32)
    adj.backward(g_cov, g_ops, g_w)
    st = adj.status()
    adj.close()
    want_g = np.zeros((len(ops), 6))
    want_w = np.zeros(len(paths))
    for i, p in enumerate(paths):
        b, n, w, h = int(p["op_begin"]), int(p["n_ops"]), int(p["width"]), int(p["height"])
        o = ops[b:b + n]
        kw = dict(s_width=float(p["s_width"]), tolerance=tolerance, transform=transform, join=join[0],
                  miter_limit=join[1])
        c64, area, s64 = oracle.adj_stroke_forward(o, w, h, **kw)
        assert st[i] == s64, (i, st[i], s64)
        off = int(p["raster_offset"]) // 4
        assert np.abs(cov[off:off + w * h].reshape(h, w) - c64).max() < COV_TOL, i
        gc = g_cov[off:off + w * h].reshape(h, w).astype(np.float64)
        gg, gw = oracle.adj_stroke_backward(o, w, h, area, gc, **kw)
        want_g[b:b + n] += gg
        want_w[i] = gw
    scale = max(np.abs(want_g).max(), np.abs(want_w).max())
    assert np.abs(g_ops - want_g).max() / scale < GRAD_TOL
    assert np.abs(g_w - want_w).max() / scale < GRAD_TOL
    return g_ops, g_w


@pytest.mark.parametrize("join", JOINS)
def test_random_strokes_match_fp64_oracle(ctx, join):
    ops, paths, cov_bytes = strokes(40 + join[0], 24)
    check(ctx, ops, paths, cov_bytes, join)


def test_example_strokes(ctx):
    fish = (Path2D().relative().pen_width(3.0).move_to(112.0, 24.0).line_to(-32.0, 24.0)
            .cubic_to(-96.0, -48.0, -96.0, 80.0, 0.0, 32.0).line_to(32.0, 24.0).line_to(-16.0, -40.0).close().finish())
    rnd = Path2D().relative().pen_width(40.0).move_to(10.0, 60.0).line_to(50.0, 0.0).line_to(0.0, -50.0).finish()
    drop = (Path2D().relative().pen_width(3.0).move_to(50.0, 34.0).cubic_to(4.0, 16.0, 16.0, 28.0, 0.0, 32.0)
            .cubic_to(-16.0, -4.0, -4.0, -16.0, 0.0, -32.0).close().finish())
    ops, paths, cov_bytes = pack_coverage([fish, rnd, drop], [128, 100, 100])
    for join in JOINS[:3]:
        g, gw = check(ctx, ops, paths, cov_bytes, join)
        assert g[0, 0] != 0.0  # fish's PenWidth op


def test_transform(ctx):
    m = (0.9, 0.15, 4.0, -0.1, 1.05, -2.0)
    ops, paths, cov_bytes = strokes(77, 10)
    ctx.set_transform(m)
    check(ctx, ops, paths, cov_bytes, JOINS[0], transform=m)


def test_wide_stroke_batch_widths(ctx):
    # the 16,384-stroke workload's shapes on 256 x 256 canvases: cubics, PenWidth first
    paths_ops, widths, clrs, side = workloads.strokes_16384(n_paths=12, side=256)
    ops, paths, cov_bytes = pack_coverage(paths_ops, [256] * len(paths_ops))
    check(ctx, ops, paths, cov_bytes, JOINS[0])
