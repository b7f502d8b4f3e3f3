"""Host batches in pipelined chunks (`ft_fill_batch` with host buffers: chunks copied in,
drawn and copied out on overlapping streams) give the same masks and statuses as the
device path and the oracle, and fall back to one pass when the layout does not allow it.
Matte8 rasters in page-locked host memory are written in place by the kernels; the rows
a figure does not reach keep the caller's bytes."""
import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, workloads
from footile_gb300.plotter import fill_batch, pack_batch

pytestmark = pytest.mark.gpu


@pytest.fixture
def chunks(ctx):
    """Force the copy pipeline's chunk count (ft_tuning.host_chunks)."""
    return lambda k: ctx.tune(host_chunks=int(k))


@pytest.fixture
def mapped_env(ctx):
    """0: page-locked host buffers used in place; 1: rasters copied; 2: ops copied too
    (ft_tuning.host_mapped)."""
    return lambda v: ctx.tune(host_mapped=int(v))


@pytest.mark.parametrize("stroke", [False, True])
def test_mapped_host_rasters(ctx, mapped_env, stroke):
    torch = pytest.importorskip("torch")
    ops, paths, nbytes = workloads.glyphs(n_paths=400, seed=41 + stroke, max_side=200)
    ops["kind"][int(paths["op_begin"][11]) + 1] = 9  # an unknown op kind in path 11
    init = np.random.default_rng(2).integers(0, 256, nbytes).astype(np.uint8)
    want = init.copy()
    oracle.fill_batch(int(stroke), _abi.NONZERO, ops, paths, _abi.MATTE8, want)
    pinned = torch.from_numpy(init.copy()).pin_memory()
    got = pinned.numpy()
    st = fill_batch(ctx, ops, paths, _abi.MATTE8, got, stroke=stroke)
    assert st[11] == _abi.ERR_ARG and (np.delete(st, 11) == 0).all()
    ok = np.ones(nbytes, bool)
    p = paths[11]
    ok[int(p["raster_offset"]):int(p["raster_offset"]) + int(p["height"]) * int(p["stride"])] = False
    assert np.array_equal(got[ok], want[ok])
    # the copy path (mapping off) writes the same bytes
    mapped_env(1)
    pinned2 = torch.from_numpy(init.copy()).pin_memory()
    got2 = pinned2.numpy()
    st2 = fill_batch(ctx, ops, paths, _abi.MATTE8, got2, stroke=stroke)
    assert np.array_equal(st2, st)
    assert np.array_equal(got2, got)


@pytest.mark.parametrize("k", [2, 3, 5])
def test_chunked_host_batch_matches_oracle(ctx, chunks, k):
    chunks(k)
    ops, paths, nbytes = workloads.glyphs(n_paths=120, seed=21 + k, max_side=160)
    ops["kind"][int(paths["op_begin"][37]) + 2] = 9  # an unknown op kind in path 37
    want = np.zeros(nbytes, np.uint8)
    want_st = oracle.fill_batch(0, _abi.NONZERO, ops, paths, _abi.MATTE8, want)
    got = np.zeros(nbytes, np.uint8)
    st = fill_batch(ctx, ops, paths, _abi.MATTE8, got)
    assert st[37] == _abi.ERR_ARG and (np.delete(st, 37) == 0).all()
    ok = np.ones(nbytes, bool)
    p = paths[37]
    ok[int(p["raster_offset"]):int(p["raster_offset"]) + int(p["height"]) * int(p["stride"])] = False
    assert np.array_equal(got[ok], want[ok])
    # the same batch again reuses every chunk's plan
    again = np.zeros(nbytes, np.uint8)
    fill_batch(ctx, ops, paths, _abi.MATTE8, again)
    assert np.array_equal(again, got)


def test_rgba_and_reversed_layout(ctx, chunks):
    chunks(3)
    rng = np.random.default_rng(5)
    sides = [int(v) for v in rng.integers(16, 120, 60)]
    per = [workloads.random_path(rng, s, int(rng.integers(4, 40))) for s in sides]
    clrs = [[int(v) for v in rng.integers(0, 128, 3)] + [200] for _ in sides]
    ops, paths, nbytes = pack_batch(per, sides, _abi.RGBA8P, clrs)
    init = np.random.default_rng(1).integers(0, 256, nbytes).astype(np.uint8)
    want = init.copy()
    oracle.fill_batch(0, _abi.NONZERO, ops, paths, _abi.RGBA8P, want)
    got = init.copy()
    fill_batch(ctx, ops, paths, _abi.RGBA8P, got)
    assert np.array_equal(got, want)
    # rasters in reverse order: not ascending, drawn in one pass
    rev = paths.copy()
    rev["raster_offset"] = paths["raster_offset"][::-1]
    rev["width"], rev["height"], rev["stride"] = paths["width"][::-1], paths["height"][::-1], paths["stride"][::-1]
    want2 = init.copy()
    oracle.fill_batch(0, _abi.NONZERO, ops, rev, _abi.RGBA8P, want2)
    got2 = init.copy()
    fill_batch(ctx, ops, rev, _abi.RGBA8P, got2)
    assert np.array_equal(got2, want2)
