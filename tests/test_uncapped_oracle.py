"""The un-capped extension in the oracle (CPU).

footile keeps at most 65,535 vertices per figure (Vid is u16, Fig::add_point ignores the
rest, fig.rs:428-442).  With `fig_cap` above that the oracle's Fig uses u32 vertex ids and
keeps up to `fig_cap` vertices; everything else is footile's algorithm.  Below the cap the
two agree exactly; above it the un-capped fill of disjoint sub-paths equals the union of
filling each alone."""
import numpy as np

import oracle
from footile_gb300 import _abi
from footile_gb300.path import Path2D


def squares(n_side, cell, pts_per_side, jitter_seed=None):
    """Disjoint squares, one sub-path each, every side split into `pts_per_side`
    collinear steps (distinct vertices that the flattening keeps)."""
    rng = np.random.default_rng(jitter_seed)
    per = []
    p = Path2D().absolute()
    for j in range(n_side):
        for i in range(n_side):
            x0, y0 = i * cell + 2.25, j * cell + 2.5
            s = cell - 5.0 + (rng.random() if jitter_seed is not None else 0.0)
            corners = [(x0, y0), (x0 + s, y0), (x0 + s, y0 + s), (x0, y0 + s)]
            q = Path2D().absolute().move_to(*corners[0])
            p.move_to(*corners[0])
            for k in range(4):
                (ax, ay), (bx, by) = corners[k], corners[(k + 1) % 4]
                for t in range(1, pts_per_side + 1):
                    x, y = ax + (bx - ax) * t / pts_per_side, ay + (by - ay) * t / pts_per_side
                    p.line_to(x, y)
                    q.line_to(x, y)
            p.close()
            per.append(q.close().finish())
    return p.finish(), per


def test_uncapped_equals_footile_below_the_cap():
    ops, _ = squares(6, 40, 50)  # 36 squares x 200 vertices
    for rule in (_abi.NONZERO, _abi.EVENODD):
        a = np.zeros((240, 240), np.uint8)
        b = np.zeros_like(a)
        oracle.fill(rule, ops, a, _abi.MATTE8)
        oracle.fill(rule, ops, b, _abi.MATTE8, fig_cap=1 << 20)
        assert np.array_equal(a, b)


def test_uncapped_keeps_every_sub_path():
    ops, per = squares(10, 30, 226, jitter_seed=3)  # 100 squares x 904 vertices = 90,400
    side = 300
    union = np.zeros((side, side), np.uint8)
    for q in per:
        m = np.zeros_like(union)
        oracle.fill(_abi.NONZERO, q, m, _abi.MATTE8)
        union = np.maximum(union, m)
    capped = np.zeros_like(union)
    oracle.fill(_abi.NONZERO, ops, capped, _abi.MATTE8)
    uncapped = np.zeros_like(union)
    oracle.fill(_abi.NONZERO, ops, uncapped, _abi.MATTE8, fig_cap=1 << 20)
    assert np.array_equal(uncapped, union)
    # footile keeps the first 65,535 vertices: the last rows of squares are missing
    assert not np.array_equal(capped, union)
    assert capped[-30:].sum() < union[-30:].sum()
    # and a cap between the two keeps a prefix of the squares
    mid = np.zeros_like(union)
    oracle.fill(_abi.NONZERO, ops, mid, _abi.MATTE8, fig_cap=80000)
    assert capped.sum() < mid.sum() < uncapped.sum()
