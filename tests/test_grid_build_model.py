"""The grid-wide figure build's formulation, restated in numpy and checked against the
oracle's sequential figure build (footile fig.rs:373-461, plotter.rs:175-224, 347).

The CUDA kernels k_gb_keep / k_gb_write (footile_gb300/csrc/ft_kernels.cu) decide every
raw vertex independently: keep (a sub-figure start, or different from the raw vertex
before it), pop (it ends a sub-figure and equals the sub-figure's first vertex), the
position as an exclusive sum of keep - pop, the cap at the first raw vertex whose
position reaches it, and the "last kept vertex of a popping sub-figure" that gives its
position to the next sub-figure.  `grid_figure` below is that formulation step for
step; these tests compare it with the oracle's Fig on line paths built to hit every
case (duplicate points, sub-figures returning to their start, single-vertex and empty
sub-figures, Close and Move in every order, the 65,535-vertex cap at many offsets)."""
import numpy as np
import pytest

import oracle
from footile_gb300 import _abi
from footile_gb300.path import PathOp, ops_array

CAP = _abi.MAX_POINTS


def raw_stream(ops):
    """Raw vertices of a Move/Line/Close/PenWidth path (identity transform, coordinates
    exact in f32) and whether each starts a sub-figure (plotter.rs:175-224)."""
    raw, rs = [], []
    prev_pc = -1
    for op in ops:
        k = int(op["kind"])
        if k in (_abi.OP_MOVE, _abi.OP_LINE):
            x, y = float(op["v"][0]), float(op["v"][1])
            raw.append((int(x * 65536), int(y * 65536)))
            rs.append(k == _abi.OP_MOVE or prev_pc in (-1, _abi.OP_CLOSE))
        if k in (_abi.OP_MOVE, _abi.OP_LINE, _abi.OP_CLOSE):
            prev_pc = k
    return np.array(raw, np.int64).reshape(-1, 2), np.array(rs, bool)


def grid_figure(raw, rs, cap):
    """Vertices and sub-figure starts of the figure, as the grid build derives them."""
    M = len(raw)
    if M == 0:
        return raw[:0], np.zeros(0, np.int64)
    idx = np.arange(M)
    R = np.maximum.accumulate(np.where(rs, idx, -1))
    assert R[0] == 0  # the first raw vertex starts a sub-figure
    same_prev = np.zeros(M, bool)
    same_prev[1:] = np.all(raw[1:] == raw[:-1], axis=1)
    keep = rs | ~same_prev
    ends = np.append(rs[1:], True)
    at_start = np.all(raw == raw[R], axis=1)
    pop = ends & at_start
    v = keep.astype(np.int64) - pop
    pos = np.concatenate([[0], np.cumsum(v)[:-1]])
    over = np.flatnonzero(pos >= cap)
    lcap = int(over[0]) if len(over) else M
    posR = pos[R]
    # the last kept vertex of a sub-figure that pops: the next kept vertex starts one
    kept = np.flatnonzero(keep)
    nxt = np.full(M, M)
    nxt[kept[:-1]] = kept[1:]
    gone = keep & at_start & ((nxt == M) | rs[np.minimum(nxt, M - 1)])
    write = keep & ~gone & (idx < lcap)
    assert np.all(pos[write] < cap)
    assert len(np.unique(pos[write])) == int(write.sum())  # one writer per position
    if lcap < M:
        count = cap - int((not rs[lcap]) and at_start[lcap - 1])
    else:
        count = int(v.sum())
    pts = np.full((max(count, int(write.sum())) + 1, 2), -1, np.int64)
    ss = np.full(len(pts), -1, np.int64)
    pts[pos[write]] = raw[write]
    ss[pos[write]] = posR[write]
    assert np.all(pts[:count] >= 0) if count else True  # every kept position is written
    return pts[:count], ss[:count]


def random_lines(rng, n_ops, grid=6, p_move=0.08, p_close=0.08, p_pw=0.02, p_back=0.1):
    """Lines on a coarse grid (many coincident points), with Moves, Closes, PenWidths
    and returns to the sub-path's start."""
    ops = []
    start = None
    for _ in range(n_ops):
        u = rng.random()
        if u < p_move or start is None:
            p = (float(rng.integers(0, grid)) * 0.25, float(rng.integers(0, grid)) * 0.25)
            ops.append(PathOp.Move(*p))
            start = p
        elif u < p_move + p_close:
            ops.append(PathOp.Close())
            if rng.random() < 0.5:
                start = None
        elif u < p_move + p_close + p_pw:
            ops.append(PathOp.PenWidth(2.0))
        elif u < p_move + p_close + p_pw + p_back:
            ops.append(PathOp.Line(*start))
        else:
            ops.append(PathOp.Line(float(rng.integers(0, grid)) * 0.25, float(rng.integers(0, grid)) * 0.25))
    return ops_array(ops)


def check(ops, cap=_abi.MAX_POINTS):
    raw, rs = raw_stream(ops)
    pts, ss = grid_figure(raw, rs, cap)
    want = oracle.fig_points(ops)
    assert len(pts) == len(want)
    np.testing.assert_array_equal(pts, want)
    # sub-figure starts: non-decreasing, each pointing at a vertex equal to its own start
    if len(ss):
        assert np.all(np.diff(ss) >= 0)
        assert np.all(ss <= np.arange(len(ss)))
        assert np.all(ss[ss] == ss)


@pytest.mark.parametrize("seed", range(40))
def test_random_line_paths(seed):
    rng = np.random.default_rng(seed)
    check(random_lines(rng, int(rng.integers(1, 400)), grid=int(rng.integers(2, 8))))


@pytest.mark.parametrize("ops", [
    [PathOp.Move(1, 1)],
    [PathOp.Close(), PathOp.Move(1, 1), PathOp.Close()],
    [PathOp.Move(1, 1), PathOp.Move(1, 1), PathOp.Move(1, 1)],
    [PathOp.Move(1, 1), PathOp.Line(1, 1), PathOp.Close(), PathOp.Line(1, 1)],
    [PathOp.Line(2, 2), PathOp.Line(2, 2), PathOp.Line(3, 2), PathOp.Line(2, 2)],
    [PathOp.Move(0, 0), PathOp.Line(1, 0), PathOp.Line(0, 0), PathOp.Move(0, 0), PathOp.Line(0, 0)],
    [PathOp.PenWidth(3.0), PathOp.Close(), PathOp.Close()],
])
def test_edge_cases(ops):
    check(ops_array(ops))


@pytest.mark.parametrize("tail", ["dup", "back", "move", "close", "line"])
@pytest.mark.parametrize("extra", [-2, -1, 0, 1, 2])
def test_cap_crossing(tail, extra):
    """Paths whose kept vertices reach 65,535 near a Move, Close, duplicate or return."""
    n = _abi.MAX_POINTS + extra
    xs = (np.arange(n) % 1000).astype(np.float32) * 0.25
    ys = (np.arange(n) // 1000).astype(np.float32) * 0.25
    ops = np.zeros(n + 4, dtype=_abi.OP_DTYPE)
    ops["kind"][0] = _abi.OP_MOVE
    ops["kind"][1:n] = _abi.OP_LINE
    ops["v"][:n, 0] = xs
    ops["v"][:n, 1] = ys
    tails = {
        "dup": [PathOp.Line(float(xs[-1]), float(ys[-1])), PathOp.Line(1.0, 1.0)],
        "back": [PathOp.Line(0.0, 0.0), PathOp.Line(0.0, 0.0)],
        "move": [PathOp.Move(0.5, 0.5), PathOp.Line(0.75, 0.5)],
        "close": [PathOp.Line(0.0, 0.0), PathOp.Close()],
        "line": [PathOp.Line(3.0, 7.0), PathOp.Line(5.0, 7.0)],
    }[tail]
    t = ops_array(tails)
    ops[n:n + len(t)] = t
    ops = ops[:n + len(t)]
    check(ops)


def test_cap_with_many_subfigures():
    """Many short sub-figures that pop, crossing the cap."""
    rng = np.random.default_rng(7)
    check(random_lines(rng, 90000, grid=40, p_move=0.2, p_close=0.2, p_back=0.2))


def cap_index(raw, rs, cap):
    """The first raw vertex whose position reaches the cap (len(raw) when none does)."""
    M = len(raw)
    if M == 0:
        return 0
    idx = np.arange(M)
    R = np.maximum.accumulate(np.where(rs, idx, -1))
    same_prev = np.zeros(M, bool)
    same_prev[1:] = np.all(raw[1:] == raw[:-1], axis=1)
    keep = rs | ~same_prev
    pop = np.append(rs[1:], True) & np.all(raw == raw[R], axis=1)
    pos = np.concatenate([[0], np.cumsum(keep.astype(np.int64) - pop)[:-1]])
    over = np.flatnonzero(pos >= cap)
    return int(over[0]) if len(over) else M


@pytest.mark.parametrize("seed", range(6))
def test_probe_prefix_completes(seed):
    """A figure built over a prefix of the ops is final once the cap falls inside the
    prefix's raw vertices (the probe of k_gb_write sets its flag only then): every
    decision before the cap vertex, and the count at it, depend on raw vertices up to it.
    Prefixes ending just before, on and after the op that reaches the cap are built and
    compared with the figure of the whole path."""
    rng = np.random.default_rng(40 + seed)
    ops = random_lines(rng, 76000, grid=300, p_move=0.04, p_close=0.04, p_back=0.05)
    raw, rs = raw_stream(ops)
    want = grid_figure(raw, rs, CAP)
    l_full = cap_index(raw, rs, CAP)
    assert l_full < len(raw), "the path must reach the cap"
    # the op that emits raw vertex l_full
    emits = np.isin(ops["kind"], [_abi.OP_MOVE, _abi.OP_LINE])
    op_of = np.flatnonzero(emits)
    j = int(op_of[l_full])
    final = 0
    for P in list(range(max(1, j - 3), min(len(ops), j + 5))) + [len(ops) - 1]:
        rp, rsp = raw_stream(ops[:P])
        if cap_index(rp, rsp, CAP) >= len(rp):
            continue  # the cap is not inside this prefix: the probe is not final
        final += 1
        pts, ss = grid_figure(rp, rsp, CAP)
        np.testing.assert_array_equal(pts, want[0])
        np.testing.assert_array_equal(ss, want[1])
    assert final >= 4
