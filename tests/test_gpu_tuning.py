"""Plan tuning and the autotuner: any tuning gives the same bytes, the autotuner picks
a plan that runs, and its cache round-trips."""
import os

import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, workloads
from footile_gb300._lib import FootileError
from footile_gb300.plotter import PreparedBatch, fill_batch

pytestmark = pytest.mark.gpu


def small_glyphs(n=600):
    return workloads.glyphs(n_paths=n, seed=13, max_side=300)


@pytest.mark.parametrize("tuning", [
    {"warp_max_side": 0, "cta_smem_bytes": 40 * 1024, "split_px": 1 << 20, "grid_per_sm": 0},
    {"warp_max_side": 64, "cta_smem_bytes": 96 * 1024, "split_px": 4096, "grid_per_sm": 2},
    {"warp_max_side": 512, "cta_smem_bytes": 64 * 1024, "split_px": 20000, "grid_per_sm": 1},
])
def test_tuning_does_not_change_results(ctx, tuning):
    ops, paths, nbytes = small_glyphs()
    want = np.zeros(nbytes, np.uint8)
    oracle.fill_batch(0, _abi.NONZERO, ops, paths, _abi.MATTE8, want, n_threads=8)
    ctx.set_tuning(tuning)
    got_t = ctx.tuning()
    assert {k: got_t[k] for k in tuning} == tuning
    assert all(got_t[k] == 0 for k in got_t if k not in tuning)  # unset knobs keep the built-in choice
    got = np.zeros(nbytes, np.uint8)
    st = fill_batch(ctx, ops, paths, _abi.MATTE8, got)
    assert (st == 0).all() and np.array_equal(got, want)
    ctx.set_tuning(None)
    assert ctx.tuning()["warp_max_side"] == 512


def test_bad_tuning_rejected(ctx):
    with pytest.raises(FootileError):
        ctx.set_tuning({"warp_max_side": 4096, "cta_smem_bytes": 0, "split_px": 0, "grid_per_sm": 0})
    with pytest.raises(FootileError):
        ctx.set_tuning({"warp_max_side": 0, "cta_smem_bytes": 1024, "split_px": 0, "grid_per_sm": 0})


def test_autotune_and_cache(ctx, tmp_path):
    torch = pytest.importorskip("torch")
    ops, paths, nbytes = small_glyphs(2000)
    ops_d = torch.from_numpy(ops.view(np.uint8)).cuda()
    ras_d = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    cache = str(tmp_path / "tuning.txt")
    t, ms = ctx.autotune(ops_d, paths, _abi.MATTE8, ras_d, cache_path=cache)
    assert ms > 0 and ctx.tuning() == t
    line = open(cache).read().split()
    # the cache keeps the batch plan's ten knobs (not the single-path fig_build)
    assert len(line) == 12 and [int(v) for v in line[1:11]] == list(t.values())[:10] and t["fig_build"] == 0
    # the tuned plan draws the same bytes
    b = PreparedBatch(ctx, paths, _abi.MATTE8)
    ras_d.zero_()
    torch.cuda.synchronize()
    b.launch(ops_d, ras_d)
    assert (b.status() == 0).all()
    want = np.zeros(nbytes, np.uint8)
    oracle.fill_batch(0, _abi.NONZERO, ops, paths, _abi.MATTE8, want, n_threads=8)
    assert np.array_equal(ras_d.cpu().numpy(), want)
    b.close()
    # a second context finds the choice in the cache without launching anything
    from footile_gb300._lib import Context
    c2 = Context(0)
    before = c2.launch_count()
    t2, ms2 = c2.autotune(ops_d, paths, _abi.MATTE8, ras_d, cache_path=cache)
    assert t2 == t and ms2 == 0.0 and c2.launch_count() == before
    c2.close()
