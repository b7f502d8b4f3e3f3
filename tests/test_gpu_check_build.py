"""The bounds-check build (-DFT_CHECK=1): the library compiled with device index checks
runs small cases of every kernel family — glyph batches (warp and CTA rasterisers), a
single large fill and stroke (figure built by one CTA and by the whole GPU, mask
compositor), ordered stroke and fill composites (tile
compositor, every tile width), Matte8 composites — with no failed check and the oracle's
bytes.  It stands in for a memory checker, which this project does not run."""
import os
import subprocess
import sys
import textwrap

import pytest

from footile_gb300 import _build

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASES = textwrap.dedent("""
    import sys
    import numpy as np
    sys.path.insert(0, ROOT); sys.path.insert(0, ROOT + "/tests")
    from footile_gb300 import _abi, _lib, workloads
    _lib.load(path=LIB)
    import ctypes, oracle
    from footile_gb300._lib import Context
    from footile_gb300.plotter import fill_batch, composite_batch, pack_batch
    from helpers import gpu_vs_oracle
    L = _lib.load()
    site, on = ctypes.c_int32(-1), ctypes.c_int32(-1)
    assert L.ft_check_failures(ctypes.byref(site), ctypes.byref(on)) == 0 and on.value == 1
    ctx = Context(0)
    for warp in (512, 0):
        ctx.tune(warp_max_side=warp)
        ops, paths, nbytes = workloads.glyphs(300, seed=71, max_side=300)
        want = np.zeros(nbytes, np.uint8); oracle.fill_batch(0, 0, ops, paths, 0, want, n_threads=8)
        got = np.zeros(nbytes, np.uint8); fill_batch(ctx, ops, paths, 0, got)
        assert np.array_equal(got, want), "glyphs"
    ctx.set_tuning(None)
    rng = np.random.default_rng(3)
    ops = workloads.random_path(rng, 1200, 200, n_sub=2)
    for fig_build in (1, 2):  # the figure (and a stroke's points and outline) on one CTA, on the whole GPU
        ctx.tune(fig_build=fig_build)
        for stroke in (False, True):
            init = rng.integers(0, 256, (1000, 1200, 4)).astype(np.uint8)
            got, want, *_ = gpu_vs_oracle(ctx, ops, 1200, 1000, fmt=_abi.RGBA8P, clr=(20, 40, 60, 200), init=init,
                                          stroke=stroke)
            assert np.array_equal(got, want), "large call"
    ctx.set_tuning(None)
    paths_ops, _, clrs, side = workloads.strokes_16384(n_paths=64, side=700)
    o, p, _ = pack_batch(paths_ops, [side] * 64, _abi.RGBA8P, clrs)
    for tw in (128, 256, 512, 1024):
        ctx.tune(tile_w=tw, band_rows=3)
        init = rng.integers(0, 256, (side, side, 4)).astype(np.uint8)
        want = init.copy(); oracle.composite(1, 0, o, p, _abi.RGBA8P, want, s_width=1.0)
        got = init.copy(); ctx.set_pen_width(1.0); composite_batch(ctx, o, p, _abi.RGBA8P, got, stroke=True)
        assert np.array_equal(got, want), f"composite {tw}"
    ctx.set_tuning(None)
    m_init = rng.integers(0, 256, (side, side)).astype(np.uint8)
    want = m_init.copy(); oracle.composite(1, 0, o, p, _abi.MATTE8, want, s_width=1.0)
    got = m_init.copy(); ctx.set_pen_width(1.0); composite_batch(ctx, o, p, _abi.MATTE8, got, stroke=True)
    assert np.array_equal(got, want), "matte8 composite"
    assert L.ft_check_failures(ctypes.byref(site), None) == 0
    print("failed check site", site.value)
    assert site.value == 0
    ctx.close()
""")


def test_check_build_runs_clean(cuda_ok, tmp_path):
    lib = _build.build_variant(str(tmp_path / "check"), ["-DFT_CHECK=1"])
    code = f"ROOT = {ROOT!r}\nLIB = {lib!r}\n" + CASES
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-3000:]
    assert "failed check site 0" in out.stdout


def test_shipped_build_has_no_checks(cuda_ok, gpu_lib):
    import ctypes
    on = ctypes.c_int32(-1)
    assert gpu_lib.ft_check_failures(None, ctypes.byref(on)) == 0 and on.value == 0
