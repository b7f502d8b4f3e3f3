"""Ordered composite: many Plotter calls on ONE raster, in order (footile's
Plotter::stroke / Plotter::fill called repeatedly, plotter.rs:339-365), on the GPU
against the oracle's calls one after another, bit-exact.  Every call composites all
pixels from its top row down (alpha 0 too, fig.rs:637-643), so the test canvases
start with random bytes and colours with small channel values, where SrcOver with
alpha 0 changes the destination."""
import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, workloads
from footile_gb300.path import PathOp, ops_array
from footile_gb300.plotter import composite_batch, pack_batch
from helpers import assert_same

pytestmark = pytest.mark.gpu


def _scene(seed, n_paths, w, h, stroke, small_colours=True):
    rng = np.random.default_rng(seed)
    paths_ops, clrs = [], []
    for i in range(n_paths):
        o = workloads.random_path(rng, max(w, h), int(rng.integers(1, 12)), close=not stroke or bool(i % 3 == 0),
                                  probs=(0.2, 0.3, 0.5))
        if stroke and i % 4 != 3:
            o = np.concatenate([ops_array([PathOp.PenWidth(float(rng.uniform(1, 12)))]), o])
        paths_ops.append(o)
        a = int(rng.integers(64, 256))
        rgb = rng.integers(0, 24 if small_colours else 256, 3)
        clrs.append([int(v) * a // 255 for v in rgb] + [a])
    ops, paths, _ = pack_batch(paths_ops, [(w, h)] * n_paths, _abi.RGBA8P, clrs)
    init = rng.integers(0, 256, (h, w, 4)).astype(np.uint8)
    return ops, paths, init


@pytest.mark.parametrize("stroke", [True, False])
@pytest.mark.parametrize("seed", range(3))
def test_composite_rgba(ctx, stroke, seed):
    ops, paths, init = _scene(40 + seed, 48, 200 + 13 * seed, 150, stroke)
    want = init.copy()
    st_o, sw_o = oracle.composite(int(stroke), _abi.NONZERO, ops, paths, _abi.RGBA8P, want, s_width=1.0)
    got = init.copy()
    ctx.set_pen_width(1.0)
    st = composite_batch(ctx, ops, paths, _abi.RGBA8P, got, stroke=stroke)
    assert (st == st_o).all()
    assert_same(got, want, f"stroke={stroke} seed={seed}")
    assert ctx.pen_width() == sw_o


@pytest.mark.parametrize("band_rows", ["1", "3", "8"])
def test_composite_band_heights(ctx, band_rows):
    ctx.tune(band_rows=int(band_rows))
    ops, paths, init = _scene(7, 30, 97, 61, True)
    want = init.copy()
    oracle.composite(1, _abi.NONZERO, ops, paths, _abi.RGBA8P, want)
    got = init.copy()
    ctx.set_pen_width(1.0)
    composite_batch(ctx, ops, paths, _abi.RGBA8P, got, stroke=True)
    assert_same(got, want, f"band rows {band_rows}")


@pytest.mark.parametrize("tile_w", [128, 256, 512, 1024])
@pytest.mark.parametrize("band_rows", [1, 3, 8])
def test_composite_tile_shapes(ctx, tile_w, band_rows):
    """Every compositor tile shape (band rows x tile width) gives the same bytes; the
    300-pixel canvas spans several tiles of 128 and 256 pixels and part of one of 512
    or 1024, so the carries between tiles and the canvas edge are exercised."""
    ctx.tune(band_rows=band_rows, tile_w=tile_w)
    ops, paths, init = _scene(17, 40, 300, 77, True)
    want = init.copy()
    oracle.composite(1, _abi.NONZERO, ops, paths, _abi.RGBA8P, want)
    got = init.copy()
    ctx.set_pen_width(1.0)
    composite_batch(ctx, ops, paths, _abi.RGBA8P, got, stroke=True)
    assert_same(got, want, f"tile {band_rows}x{tile_w}")


@pytest.mark.parametrize("w", [101, 300])
def test_composite_canvas_staging(ctx, w):
    """Rows 404 bytes apart (not a multiple of 16) cannot be described by a TMA tensor
    map: the compositor stages the canvas with plain loads and stores; 1,200-byte rows
    go through TMA.  Both give the oracle's bytes."""
    ops, paths, init = _scene(23, 36, w, 90, False)
    want = init.copy()
    oracle.composite(0, _abi.EVENODD, ops, paths, _abi.RGBA8P, want)
    got = init.copy()
    composite_batch(ctx, ops, paths, _abi.RGBA8P, got, rule=_abi.EVENODD)
    assert_same(got, want, f"width {w}")


def test_composite_matte8_evenodd(ctx):
    ops, paths, _ = _scene(3, 40, 120, 90, False)
    init = np.random.default_rng(1).integers(0, 256, (90, 120)).astype(np.uint8)
    want = init.copy()
    oracle.composite(0, _abi.EVENODD, ops, paths, _abi.MATTE8, want)
    got = init.copy()
    composite_batch(ctx, ops, paths, _abi.MATTE8, got, rule=_abi.EVENODD)
    assert_same(got, want, "matte8 even-odd")


def test_composite_pool_grows(ctx):
    # a tiny first edge pool forces the build to overflow and run again
    ctx.tune(pool_edges=500)
    ops, paths, init = _scene(11, 24, 150, 110, True)
    want = init.copy()
    oracle.composite(1, _abi.NONZERO, ops, paths, _abi.RGBA8P, want)
    got = init.copy()
    ctx.set_pen_width(1.0)
    st = composite_batch(ctx, ops, paths, _abi.RGBA8P, got, stroke=True)
    assert (st == 0).all()
    assert_same(got, want, "pool growth")


def test_composite_device_buffers(ctx):
    torch = pytest.importorskip("torch")
    ops, paths, init = _scene(21, 64, 256, 256, True, small_colours=False)
    want = init.copy()
    _, sw = oracle.composite(1, _abi.NONZERO, ops, paths, _abi.RGBA8P, want)
    from footile_gb300.plotter import pen_width_chain
    paths["s_width"], _ = pen_width_chain(ops, paths, 1.0)
    ops_d = torch.from_numpy(ops.view(np.uint8)).cuda()
    ras_d = torch.from_numpy(init).cuda()
    composite_batch(ctx, ops_d, paths, _abi.RGBA8P, ras_d, stroke=True)
    assert_same(ras_d.cpu().numpy(), want, "device composite")


@pytest.mark.parametrize("init_kind", ["zero", "random"])
def test_strokes_16384_prefix_full_canvas(ctx, init_kind):
    """The benchmark's ordered stroke composite at full canvas size: the first 1,024 of
    the 16,384 strokes (8..64 cubics, width 1..12, Miter(4), alpha 64..255) drawn in
    order onto the 2048x2048 Rgba8p canvas, against the oracle's Plotter::stroke calls
    one after another (the oracle composites every pixel from each call's top row down:
    about 24 s on one core).  A random initial canvas also exercises the alpha-0
    composites of every call."""
    torch = pytest.importorskip("torch")
    from footile_gb300.plotter import pen_width_chain
    k = 1024
    paths_ops, _, clrs, side = workloads.strokes_16384()
    ops, paths, _ = pack_batch(paths_ops[:k], [side] * k, _abi.RGBA8P, clrs[:k])
    paths["s_width"], _ = pen_width_chain(ops, paths, 1.0)
    if init_kind == "zero":
        init = np.zeros((side, side, 4), np.uint8)
    else:
        init = np.random.default_rng(6).integers(0, 256, (side, side, 4)).astype(np.uint8)
    want = init.copy()
    st_o, _ = oracle.composite(1, _abi.NONZERO, ops, paths, _abi.RGBA8P, want, s_width=1.0,
                               join=_abi.JOIN_MITER, miter_limit=4.0)
    ctx.set_join(_abi.JOIN_MITER, 4.0)
    ops_d = torch.from_numpy(ops.view(np.uint8)).cuda()
    ras_d = torch.from_numpy(init).cuda()
    st = composite_batch(ctx, ops_d, paths, _abi.RGBA8P, ras_d, stroke=True)
    assert (st == st_o).all()
    assert_same(ras_d.cpu().numpy(), want, f"{k} strokes on {side}x{side} ({init_kind} canvas)")


@pytest.mark.parametrize("w,h", [(1, 1), (5, 3), (130, 1), (3, 200), (1030, 9)])
def test_composite_ragged_canvases(ctx, w, h):
    """Canvases narrower than a tile, one row or one column high, and a width just past a
    1,024-pixel tile: the tile compositor's edges (partial tiles, rows past the canvas,
    chunks past its right edge) against the oracle, Rgba8p on random bytes."""
    rng = np.random.default_rng(w * 1000 + h)
    paths_ops, clrs = [], []
    for i in range(12):
        o = workloads.random_path(rng, max(w, h) + 4, int(rng.integers(1, 8)), close=bool(i % 2))
        o["v"] -= 2.0  # some coordinates left of and above the canvas
        paths_ops.append(o)
        a = int(rng.integers(1, 256))
        clrs.append([int(v) * a // 255 for v in rng.integers(0, 256, 3)] + [a])
    ops, paths, _ = pack_batch(paths_ops, [(w, h)] * len(paths_ops), _abi.RGBA8P, clrs)
    init = rng.integers(0, 256, (h, w, 4)).astype(np.uint8)
    for stroke in (False, True):
        want = init.copy()
        oracle.composite(int(stroke), _abi.NONZERO, ops, paths, _abi.RGBA8P, want, s_width=1.0)
        got = init.copy()
        ctx.set_pen_width(1.0)
        composite_batch(ctx, ops, paths, _abi.RGBA8P, got, stroke=stroke)
        assert_same(got, want, f"{w}x{h} stroke={stroke}")


def test_composite_empty_and_offcanvas_calls(ctx):
    """Calls with no ops, calls whose figures lie wholly below, right of or above the
    canvas, and an empty call list: only footile's alpha-0 composites of the calls that
    reach a row change the canvas."""
    rng = np.random.default_rng(99)
    w, h = 300, 120
    square = lambda x, y: ops_array([PathOp.Move(x, y), PathOp.Line(x + 20, y), PathOp.Line(x + 20, y + 20),
                                     PathOp.Line(x, y + 20), PathOp.Close()])
    paths_ops = [ops_array([]), square(10, 500), square(900, 10), square(10, -400), square(40, 30),
                 ops_array([PathOp.Move(5, 5)]), square(-30, 60)]
    clrs = [[10, 5, 3, 200]] * len(paths_ops)
    ops, paths, _ = pack_batch(paths_ops, [(w, h)] * len(paths_ops), _abi.RGBA8P, clrs)
    init = rng.integers(0, 24, (h, w, 4)).astype(np.uint8)
    want = init.copy()
    oracle.composite(0, _abi.NONZERO, ops, paths, _abi.RGBA8P, want)
    got = init.copy()
    composite_batch(ctx, ops, paths, _abi.RGBA8P, got)
    assert_same(got, want, "empty and off-canvas calls")
    none = init.copy()
    composite_batch(ctx, ops[:0], paths[:0], _abi.RGBA8P, none)
    assert_same(none, init, "no calls")
