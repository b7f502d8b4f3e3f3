"""The grid-wide stroke build's point formulation, restated in numpy and checked against
the oracle's sequential stroker (footile stroker.rs:204-236).

The CUDA kernels k_gs_keep / k_gs_write / k_gs_subs (footile_gb300/csrc/ft_kernels.cu)
decide every raw stroke point on its own: it starts a sub-stroke when it is the first
point or a close came before it (since the point before), it is kept when it starts a
sub-stroke or differs in x or y from the raw point before it, its position is an
exclusive sum of the kept flags and its sub-stroke an exclusive sum of the start flags;
points at or past 65,535 are dropped, a start point writes the joined flag of the last
close before it into the sub-stroke before, and the last sub-stroke takes its joined and
done flags from the closes after the last point written.  `grid_points` below is that
formulation step for step; the tests compare it with the oracle's Stroke on paths built
to hit every case (coincident points, Close and Move in every order, empty sub-paths,
pen-width changes, the point cap with closes after it)."""
import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, workloads
from footile_gb300.path import PathOp, ops_array

CAP = _abi.MAX_POINTS


def grid_points(ev, cap=CAP, ev_all=None):
    """Kept stroke points (x, y, width) and sub-strokes (start, points, joined, done).
    `ev_all` (a stream that `ev` is a prefix of): the last sub-stroke's flags come from
    its closes, as the probe takes them from the ops of the whole path."""
    is_pt = ev[:, 3] == 0
    raw = ev[is_pt, :3]
    M = len(raw)
    if M == 0:
        return raw[:0], np.array([[0, 0, 0, 0]], np.int32)
    # per raw point: a close since the raw point before, and the last close's joined flag
    ev_idx = np.flatnonzero(is_pt)
    starts = np.zeros(M, bool)
    joined_before = np.zeros(M, np.int32)
    for k in range(M):
        lo = ev_idx[k - 1] + 1 if k else 0
        closes = ev[lo:ev_idx[k], 3]
        if k == 0 or len(closes):
            starts[k] = True
        if len(closes):
            joined_before[k] = int(closes[-1]) - 1
    same = np.zeros(M, bool)
    same[1:] = (raw[1:, 0] == raw[:-1, 0]) & (raw[1:, 1] == raw[:-1, 1])
    keep = starts | ~same
    pos = np.concatenate([[0], np.cumsum(keep)[:-1]])
    sid = np.concatenate([[0], np.cumsum(starts)[:-1]])
    written = keep & (pos < cap)
    count = int(written.sum())
    pts = np.zeros((count, 3), np.float32)
    pts[pos[written]] = raw[written]
    new_sub = written & starts
    n_subs = int(sid[new_sub].max()) + 1
    subs = np.zeros((n_subs, 4), np.int32)
    subs[sid[new_sub], 0] = pos[new_sub]
    later = new_sub & (sid > 0)
    subs[sid[later] - 1, 2] = joined_before[later]
    subs[:-1, 3] = 1
    subs[:-1, 1] = np.diff(subs[:, 0])
    subs[-1, 1] = count - subs[-1, 0]
    # the last sub-stroke: the closes after the last point written
    last = int(ev_idx[np.flatnonzero(written)[-1]])
    tail = (ev if ev_all is None else ev_all)[last + 1:, 3]
    tail = tail[tail > 0]
    if len(tail):
        subs[-1, 2] = int(tail[-1]) - 1
        subs[-1, 3] = 1
    return pts, subs


def check(ops, s_width=1.0, **params):
    ev, want_pts, want_subs = oracle.stroke_points(ops, s_width=s_width, **params)
    pts, subs = grid_points(ev)
    assert len(pts) == len(want_pts)
    np.testing.assert_array_equal(pts, want_pts)
    np.testing.assert_array_equal(subs, want_subs)
    return len(pts), len(subs)


def random_ops(rng, n_ops, grid=5):
    """Lines on a coarse grid (many coincident points), Moves, Closes and pen widths."""
    ops = []
    for _ in range(n_ops):
        u = rng.random()
        p = (float(rng.integers(0, grid)), float(rng.integers(0, grid)))
        if u < 0.12:
            ops.append(PathOp.Move(*p))
        elif u < 0.24:
            ops.append(PathOp.Close())
        elif u < 0.28:
            ops.append(PathOp.PenWidth(float(rng.integers(1, 6))))
        else:
            ops.append(PathOp.Line(*p))
    return ops_array(ops)


@pytest.mark.parametrize("seed", range(40))
def test_random_line_strokes(seed):
    rng = np.random.default_rng(500 + seed)
    check(random_ops(rng, int(rng.integers(1, 300)), grid=int(rng.integers(2, 7))))


@pytest.mark.parametrize("seed", range(12))
def test_random_curve_strokes(seed):
    rng = np.random.default_rng(900 + seed)
    ops = workloads.random_path(rng, 200, int(rng.integers(1, 40)), n_sub=int(rng.integers(1, 5)),
                                close=bool(seed % 2))
    pw = ops_array([PathOp.PenWidth(float(rng.uniform(0.5, 14.0)))])
    check(np.concatenate([pw, ops]), tolerance=float(rng.choice([0.1, 0.3, 1.0])))


@pytest.mark.parametrize("ops", [
    [],
    [PathOp.Move(5, 5)],
    [PathOp.Close(), PathOp.Close()],
    [PathOp.Move(5, 5), PathOp.Close()],
    [PathOp.Move(5, 5), PathOp.Line(5, 5), PathOp.Close(), PathOp.Line(5, 5)],
    [PathOp.Move(1, 1), PathOp.Line(4, 1), PathOp.Close(), PathOp.Move(1, 1), PathOp.Line(1, 1)],
    [PathOp.Move(1, 1), PathOp.Line(4, 1), PathOp.Close(), PathOp.Line(6, 6), PathOp.Close(), PathOp.Move(2, 2)],
    [PathOp.PenWidth(3.0), PathOp.Move(1, 1), PathOp.PenWidth(5.0), PathOp.Line(1, 1), PathOp.Line(3, 3)],
])
def test_edge_cases(ops):
    check(ops_array(ops))


@pytest.mark.parametrize("tail", ["close", "close_move", "move_close", "dup", "none"])
@pytest.mark.parametrize("extra", [-2, 0, 2])
def test_point_cap(tail, extra):
    """More than 65,535 stroke points: footile keeps the first 65,535, and closes after
    the cap still set the last sub-stroke's joined and done flags."""
    n = CAP + extra
    ops = np.zeros(n, dtype=_abi.OP_DTYPE)
    ops["kind"][0] = _abi.OP_MOVE
    ops["kind"][1:] = _abi.OP_LINE
    ops["v"][:, 0] = (np.arange(n) % 1000).astype(np.float32)
    ops["v"][:, 1] = (np.arange(n) // 1000).astype(np.float32)
    tails = {
        "close": [PathOp.Close()],
        "close_move": [PathOp.Close(), PathOp.Move(3, 3), PathOp.Line(7, 3)],
        "move_close": [PathOp.Move(3, 3), PathOp.Line(7, 3), PathOp.Close()],
        "dup": [PathOp.Line(float((n - 1) % 1000), float((n - 1) // 1000)), PathOp.Close()],
        "none": [],
    }[tail]
    ops = np.concatenate([ops, ops_array(tails)]) if tails else ops
    n_pts, _ = check(ops)
    if extra >= 0:
        assert n_pts == CAP


def kept_count(ev):
    """Stroke points a stream keeps before the cap applies."""
    raw = ev[ev[:, 3] == 0]
    if not len(raw):
        return 0
    ev_idx = np.flatnonzero(ev[:, 3] == 0)
    starts = np.array([k == 0 or bool((ev[(ev_idx[k - 1] + 1 if k else 0):ev_idx[k], 3] > 0).any())
                       for k in range(len(raw))])
    same = np.zeros(len(raw), bool)
    same[1:] = (raw[1:, 0] == raw[:-1, 0]) & (raw[1:, 1] == raw[:-1, 1])
    return int((starts | ~same).sum())


@pytest.mark.parametrize("tail", ["close_move", "line", "move_close"])
def test_probe_prefix_completes(tail):
    """The stroke points over a prefix of the ops are final once the prefix keeps more
    than 65,535 (the probe of k_gs_keep sets its flag only then): the points and
    sub-stroke starts come from the prefix, the last sub-stroke's joined and done flags
    from the closes of the whole path.  Prefixes ending around the op whose point is the
    65,536th kept are compared with the whole path."""
    rng = np.random.default_rng(77)
    n = CAP + 1200
    ops = np.zeros(n, dtype=_abi.OP_DTYPE)
    ops["kind"][:] = _abi.OP_LINE
    ops["kind"][rng.integers(0, n, 300)] = _abi.OP_MOVE
    ops["kind"][rng.integers(0, n, 300)] = _abi.OP_CLOSE
    ops["kind"][0] = _abi.OP_MOVE
    ops["v"][:, 0] = rng.integers(0, 200, n).astype(np.float32)
    ops["v"][:, 1] = rng.integers(0, 200, n).astype(np.float32)
    extra = {"close_move": [PathOp.Close(), PathOp.Move(3, 3), PathOp.Close()],
             "line": [PathOp.Line(4, 4), PathOp.Line(8, 4)],
             "move_close": [PathOp.Move(3, 3), PathOp.Close()]}[tail]
    ops = np.concatenate([ops, ops_array(extra)])
    ev, want_pts, want_subs = oracle.stroke_points(ops)
    assert len(want_pts) == CAP
    # the op that emits the 65,536th kept point
    emits = np.flatnonzero(np.isin(ops["kind"], [_abi.OP_MOVE, _abi.OP_LINE]))
    lo, hi = 1, len(ops)
    while lo < hi:  # the shortest prefix keeping more than the cap
        mid = (lo + hi) // 2
        if kept_count(oracle.stroke_points(ops[:mid])[0]) > CAP:
            hi = mid
        else:
            lo = mid
            lo += 1
    assert ops["kind"][lo - 1] in (_abi.OP_MOVE, _abi.OP_LINE) and lo - 1 in emits
    final = 0
    for P in list(range(lo - 3, min(lo + 4, len(ops) + 1))) + [len(ops)]:
        ev_p = oracle.stroke_points(ops[:P])[0]
        assert np.array_equal(ev_p, ev[:len(ev_p)])
        if kept_count(ev_p) <= CAP:
            continue  # the probe is not final
        final += 1
        pts, subs = grid_points(ev_p, ev_all=ev)
        np.testing.assert_array_equal(pts, want_pts)
        np.testing.assert_array_equal(subs, want_subs)
    assert final >= 4
