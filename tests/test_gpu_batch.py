"""Batched fills (one persistent launch over many independent Plotter calls)
against the oracle, bit-exact; host-resident and device-resident buffers."""
import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, workloads
from footile_gb300.plotter import fill_batch
from helpers import assert_same

pytestmark = pytest.mark.gpu


def _compare_paths(got, want, paths, which):
    for i in which:
        d = paths[i]
        a = got[d["raster_offset"]: d["raster_offset"] + d["stride"] * d["height"]]
        b = want[d["raster_offset"]: d["raster_offset"] + d["stride"] * d["height"]]
        a = a.reshape(d["height"], d["stride"])[:, : d["width"]]
        b = b.reshape(d["height"], d["stride"])[:, : d["width"]]
        assert_same(a, b, f"path {i} ({d['n_ops']} ops, {d['width']}x{d['height']})")


@pytest.mark.parametrize("warp", ["512", "0"])
@pytest.mark.parametrize("rule", [_abi.NONZERO, _abi.EVENODD])
def test_glyph_batch_host(ctx, rule, warp):
    ctx.tune(warp_max_side=int(warp))
    ops, paths, nbytes = workloads.glyphs(3000, seed=31)
    want = np.zeros(nbytes, np.uint8)
    st_o = oracle.fill_batch(0, rule, ops, paths, _abi.MATTE8, want, n_threads=8)
    got = np.zeros(nbytes, np.uint8)
    st = fill_batch(ctx, ops, paths, _abi.MATTE8, got, rule=rule)
    assert (st == st_o).all()
    if not np.array_equal(got, want):
        _compare_paths(got, want, paths, range(len(paths)))


def _mismatching_paths(got, want, paths):
    """Indices of the paths whose raster bytes differ (rasters back to back)."""
    bad = np.flatnonzero(got != want)
    if len(bad) == 0:
        return np.zeros(0, np.int64)
    return np.unique(np.searchsorted(paths["raster_offset"].astype(np.int64), bad, side="right") - 1)


def test_glyph_batch_device_full_size(ctx):
    """The full 65,536-path glyph workload of the benchmark, on the device: every path's
    mask bit-exact against the oracle (rows above a path's top vertex keep the initial
    byte on both sides)."""
    torch = pytest.importorskip("torch")
    import os
    ops, paths, nbytes = workloads.glyphs_65536()
    init = 0x5A
    ops_d = torch.from_numpy(ops.view(np.uint8)).cuda()
    ras_d = torch.full((nbytes,), init, dtype=torch.uint8, device="cuda")
    st = fill_batch(ctx, ops_d, paths, _abi.MATTE8, ras_d)
    assert (st == 0).all()
    got = ras_d.cpu().numpy()
    want = np.full(nbytes, init, np.uint8)
    st_o = oracle.fill_batch(0, _abi.NONZERO, ops, paths, _abi.MATTE8, want, n_threads=os.cpu_count() or 8)
    assert (st_o == 0).all()
    bad = _mismatching_paths(got, want, paths)
    if len(bad):
        _compare_paths(got, want, paths, bad[:1])
    assert len(bad) == 0, f"{len(bad)} of {len(paths)} paths differ"


def test_glyph_batch_prepared_full_size(ctx):
    """The benchmark's timed object: a prepared batch (CUDA graph replay) of the
    65,536 glyphs, launched twice onto the same rasters; every mask bit-exact."""
    torch = pytest.importorskip("torch")
    import os
    from footile_gb300.plotter import PreparedBatch
    ops, paths, nbytes = workloads.glyphs_65536()
    ops_d = torch.from_numpy(ops.view(np.uint8)).cuda()
    ras_d = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
    b = PreparedBatch(ctx, paths, _abi.MATTE8)
    b.launch(ops_d, ras_d)
    b.launch(ops_d, ras_d)
    assert (b.status() == 0).all()
    b.close()
    got = ras_d.cpu().numpy()
    want = np.zeros(nbytes, np.uint8)
    oracle.fill_batch(0, _abi.NONZERO, ops, paths, _abi.MATTE8, want, n_threads=os.cpu_count() or 8)
    bad = _mismatching_paths(got, want, paths)
    assert len(bad) == 0, f"{len(bad)} of {len(paths)} paths differ"


def test_batch_rgba_regions(ctx):
    rng = np.random.default_rng(9)
    paths_ops, sizes, clrs = [], [], []
    for i in range(64):
        side = int(rng.integers(8, 120))
        paths_ops.append(workloads.random_path(rng, side, int(rng.integers(3, 40))))
        sizes.append((side, int(rng.integers(8, 120))))
        a = int(rng.integers(1, 256))
        clrs.append([int(v) for v in rng.integers(0, a + 1, 3)] + [a])
    from footile_gb300.plotter import pack_batch
    ops, paths, nbytes = pack_batch(paths_ops, sizes, _abi.RGBA8P, clrs)
    init = rng.integers(0, 256, nbytes).astype(np.uint8)
    want = init.copy()
    oracle.fill_batch(0, _abi.NONZERO, ops, paths, _abi.RGBA8P, want, n_threads=4)
    got = init.copy()
    fill_batch(ctx, ops, paths, _abi.RGBA8P, got)
    assert_same(got, want, "rgba batch")


def test_plan_reuse_and_invalidation(ctx):
    # the same batch twice reuses its plan; a changed descriptor, a different batch
    # and a single call in between must all replan
    from footile_gb300.plotter import Plotter
    a_ops, a_paths, a_bytes = workloads.glyphs(n_paths=300, seed=31, max_side=200)
    b_ops, b_paths, b_bytes = workloads.glyphs(n_paths=300, seed=32, max_side=200)

    def run(ops, paths, nbytes):
        want = np.zeros(nbytes, np.uint8)
        oracle.fill_batch(0, _abi.NONZERO, ops, paths, _abi.MATTE8, want, n_threads=8)
        got = np.zeros(nbytes, np.uint8)
        assert (fill_batch(ctx, ops, paths, _abi.MATTE8, got) == 0).all()
        assert np.array_equal(got, want)
    run(a_ops, a_paths, a_bytes)
    run(a_ops, a_paths, a_bytes)
    run(b_ops, b_paths, b_bytes)
    run(a_ops, a_paths, a_bytes)
    c_paths = a_paths.copy()
    c_paths[0]["height"] = max(1, int(c_paths[0]["height"]) // 2)  # same length, one descriptor changed
    run(a_ops, c_paths, a_bytes)
    single = np.zeros((64, 64), np.uint8)
    Plotter(single, context=ctx).fill(_abi.NONZERO, workloads.random_path(np.random.default_rng(3), 64, 10))
    run(a_ops, a_paths, a_bytes)

