"""Seeded synthetic scenes with the shapes of the benchmark configurations.

All paths are built in absolute coordinates: move_to(P0), segments, [close]
(footile src/path.rs:66-69).  numpy's PCG64 generator makes them reproducible on
any host.

  single_path_256   one closed path, 64 mixed segments, 256x256 canvas
  scene_4096        one 4096x4096 canvas, 1,000 sub-paths x 100 mixed segments
  glyphs_65536      65,536 closed glyph-like paths, 4..400 segments (log-uniform),
                    70% quad / 20% cubic / 10% line, canvas side 16..256 (log-uniform)
  cubics_1024       1,024 closed paths of 32 cubics on 128x128 canvases
  strokes_16384     16,384 open paths of 8..64 cubics on one 2048x2048 canvas,
                    pen width 1..12, ordered composite colours
"""
import numpy as np

from . import _abi
from .plotter import pack_batch

SEG_LINE, SEG_QUAD, SEG_CUBIC = 0, 1, 2


def _ops_from_segments(starts, seg_type, coords, close):
    """Vectorised op building for many sub-paths.

    starts:   (S, 2) move_to points
    seg_type: list of (n_s,) arrays of segment types per sub-path
    coords:   list of (n_s, 6) arrays of coordinates per sub-path
    close:    bool, add a Close op after each sub-path
    Returns an array of ft_op records for all sub-paths back to back.
    """
    n_sub = len(starts)
    counts = np.array([len(t) for t in seg_type], dtype=np.int64)
    per = counts + 1 + (1 if close else 0)
    total = int(per.sum())
    ops = np.zeros(total, dtype=_abi.OP_DTYPE)
    begin = np.concatenate([[0], np.cumsum(per)[:-1]])
    ops["kind"][begin] = _abi.OP_MOVE
    ops["v"][begin, 0] = starts[:, 0]
    ops["v"][begin, 1] = starts[:, 1]
    if counts.sum():
        seg_idx = np.concatenate([b + 1 + np.arange(c) for b, c in zip(begin, counts)])
        t = np.concatenate(seg_type)
        cc = np.concatenate(coords).astype(np.float32)
        kind = np.where(t == SEG_LINE, _abi.OP_LINE, np.where(t == SEG_QUAD, _abi.OP_QUAD, _abi.OP_CUBIC))
        ops["kind"][seg_idx] = kind
        v = np.zeros((len(t), 6), np.float32)
        # line: end point; quad: control + end; cubic: two controls + end
        v[t == SEG_LINE, 0:2] = cc[t == SEG_LINE, 0:2]
        v[t == SEG_QUAD, 0:4] = cc[t == SEG_QUAD, 0:4]
        v[t == SEG_CUBIC, 0:6] = cc[t == SEG_CUBIC, 0:6]
        ops["v"][seg_idx] = v
    if close:
        ops["kind"][begin + per - 1] = _abi.OP_CLOSE
    return ops, begin, per


def _mixed_types(rng, n, probs=(1 / 3, 1 / 3, 1 / 3)):
    u = rng.random(n)
    p_line, p_quad = probs[0], probs[1]
    return np.where(u < p_line, SEG_LINE, np.where(u < p_line + p_quad, SEG_QUAD, SEG_CUBIC)).astype(np.int8)


def single_path_256(seed=1):
    """One closed path of 64 mixed segments on a 256x256 canvas, and a colour."""
    rng = np.random.default_rng(seed)
    t = _mixed_types(rng, 64)
    coords = (rng.random((64, 6)) * 256).astype(np.float32)
    start = (rng.random((1, 2)) * 256).astype(np.float32)
    ops, _, _ = _ops_from_segments(start, [t], [coords], close=True)
    clr = np.concatenate([rng.integers(0, 256, 3), [255]]).astype(np.uint8)
    return ops, 256, 256, clr


def scene_4096(seed=2, n_sub=1000, n_seg=100, side=4096):
    """One self-intersecting scene: `n_sub` closed sub-paths of `n_seg` mixed segments."""
    rng = np.random.default_rng(seed)
    starts = (rng.random((n_sub, 2)) * side).astype(np.float32)
    types = [_mixed_types(rng, n_seg) for _ in range(n_sub)]
    coords = [(rng.random((n_seg, 6)) * side).astype(np.float32) for _ in range(n_sub)]
    ops, _, _ = _ops_from_segments(starts, types, coords, close=True)
    clr = np.concatenate([rng.integers(0, 256, 3), [255]]).astype(np.uint8)
    return ops, side, side, clr


def glyphs(n_paths=65536, seed=3, min_seg=4, max_seg=400, min_side=16, max_side=256):
    """Uneven glyph-like closed paths, each on its own square canvas.

    Returns (ops, paths, raster_bytes) ready for `fill_batch` (Matte8).
    """
    rng = np.random.default_rng(seed)
    n_seg = np.rint(np.exp(rng.uniform(np.log(min_seg), np.log(max_seg), n_paths))).astype(np.int64)
    side = np.rint(np.exp(rng.uniform(np.log(min_side), np.log(max_side), n_paths))).astype(np.int64)
    total_seg = int(n_seg.sum())
    u = rng.random(total_seg)
    t_all = np.where(u < 0.7, SEG_QUAD, np.where(u < 0.9, SEG_CUBIC, SEG_LINE)).astype(np.int8)
    seg_side = np.repeat(side, n_seg).astype(np.float32)
    c_all = (rng.random((total_seg, 6)).astype(np.float32) * seg_side[:, None]).astype(np.float32)
    starts = (rng.random((n_paths, 2)).astype(np.float32) * side[:, None].astype(np.float32)).astype(np.float32)
    # fast vectorised op layout: [move, segs..., close] per path
    per = n_seg + 2
    total = int(per.sum())
    ops = np.zeros(total, dtype=_abi.OP_DTYPE)
    begin = np.concatenate([[0], np.cumsum(per)[:-1]]).astype(np.int64)
    ops["kind"][begin] = _abi.OP_MOVE
    ops["v"][begin, 0:2] = starts
    seg_pos = np.repeat(begin + 1, n_seg) + (np.arange(total_seg) - np.repeat(np.cumsum(n_seg) - n_seg, n_seg))
    kind = np.where(t_all == SEG_LINE, _abi.OP_LINE, np.where(t_all == SEG_QUAD, _abi.OP_QUAD, _abi.OP_CUBIC))
    ops["kind"][seg_pos] = kind
    v = np.zeros((total_seg, 6), np.float32)
    m = t_all == SEG_LINE
    v[m, 0:2] = c_all[m, 0:2]
    m = t_all == SEG_QUAD
    v[m, 0:4] = c_all[m, 0:4]
    m = t_all == SEG_CUBIC
    v[m] = c_all[m]
    ops["v"][seg_pos] = v
    ops["kind"][begin + per - 1] = _abi.OP_CLOSE
    # path descriptors: canvases back to back, rows padded to 4 bytes
    paths = np.zeros(n_paths, dtype=_abi.PATH_DTYPE)
    stride = ((side + 3) // 4) * 4
    sizes = stride * side
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    paths["op_begin"] = begin
    paths["n_ops"] = per
    paths["width"] = side
    paths["height"] = side
    paths["raster_offset"] = offs
    paths["stride"] = stride
    paths["s_width"] = 1.0
    return ops, paths, int(sizes.sum())


def glyphs_65536(seed=3):
    return glyphs(65536, seed)


def cubics_1024(seed=4, n_paths=1024, n_seg=32, side=128):
    """Closed paths of `n_seg` cubics with control points in [16, 112)."""
    rng = np.random.default_rng(seed)
    starts = (16 + rng.random((n_paths, 2)) * 96).astype(np.float32)
    types = [np.full(n_seg, SEG_CUBIC, np.int8) for _ in range(n_paths)]
    coords = [(16 + rng.random((n_seg, 6)) * 96).astype(np.float32) for _ in range(n_paths)]
    paths_ops = []
    for i in range(n_paths):
        o, _, _ = _ops_from_segments(starts[i:i + 1], [types[i]], [coords[i]], close=True)
        paths_ops.append(o)
    ops, paths, nbytes = pack_batch(paths_ops, [side] * n_paths)
    return ops, paths, nbytes


def cubics_1024_coverage(seed=4, target_seed=5, n_paths=1024, n_seg=32, side=128):
    """The closed-cubic batch of `cubics_1024` packed for the coverage adjoint: one f32
    coverage plane per path, and a target of uniform [0, 1) values (seed 5) for the
    L2 loss sum((cov - target)^2).  Returns (ops, paths, cov_bytes, target)."""
    from .adjoint import pack_coverage
    ops, paths, _ = cubics_1024(seed, n_paths, n_seg, side)
    per_path = [ops[p["op_begin"]:p["op_begin"] + p["n_ops"]] for p in paths]
    ops_c, paths_c, cov_bytes = pack_coverage(per_path, [side] * n_paths)
    target = np.random.default_rng(target_seed).random(cov_bytes // 4, dtype=np.float32)
    return ops_c, paths_c, cov_bytes, target


def strokes_16384(seed=6, n_paths=16384, side=2048, min_seg=8, max_seg=64):
    """Open cubic paths with a PenWidth op each, premultiplied colours, one canvas."""
    rng = np.random.default_rng(seed)
    n_seg = rng.integers(min_seg, max_seg + 1, n_paths)
    widths = rng.uniform(1.0, 12.0, n_paths).astype(np.float32)
    rgb = rng.integers(0, 256, (n_paths, 3))
    alpha = rng.integers(64, 256, n_paths)
    clrs = np.zeros((n_paths, 4), np.uint8)
    clrs[:, :3] = (rgb * alpha[:, None] + 127) // 255
    clrs[:, 3] = alpha
    paths_ops = []
    for i in range(n_paths):
        start = (rng.random((1, 2)) * side).astype(np.float32)
        coords = (rng.random((n_seg[i], 6)) * side).astype(np.float32)
        o, _, _ = _ops_from_segments(start, [np.full(n_seg[i], SEG_CUBIC, np.int8)], [coords], close=False)
        pw = np.zeros(1, dtype=_abi.OP_DTYPE)
        pw["kind"] = _abi.OP_PEN_WIDTH
        pw["v"][0, 0] = widths[i]
        paths_ops.append(np.concatenate([pw, o]))
    return paths_ops, widths, clrs, side


def random_path(rng, side, n_seg, probs=(1 / 3, 1 / 3, 1 / 3), close=True, n_sub=1):
    """A random path of `n_sub` sub-paths with coordinates in [0, side)."""
    starts = (rng.random((n_sub, 2)) * side).astype(np.float32)
    types = [_mixed_types(rng, n_seg, probs) for _ in range(n_sub)]
    coords = [(rng.random((n_seg, 6)) * side).astype(np.float32) for _ in range(n_sub)]
    ops, _, _ = _ops_from_segments(starts, types, coords, close=close)
    return ops
