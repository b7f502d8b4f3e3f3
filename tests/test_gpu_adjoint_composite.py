"""Differentiable ordered composite of strokes on one canvas on the GPU
(ft_srcover_forward / ft_srcover_backward, and ft_stroke_composite_forward / _backward,
which covers the strokes chunk by chunk and recomputes them in the backward) against
the FP64 chain: the composited canvas within 1e-4, gradients of the op floats, pen
widths and initial canvas within 2e-4 of the largest entry, for every chunk size."""
import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, workloads
from footile_gb300._lib import FootileError
from footile_gb300.adjoint import (StrokeComposite, pack_coverage, srcover_backward, srcover_forward,
                                   stroke_composite_grads)

pytestmark = pytest.mark.gpu


def test_srcover_adjoint_against_numpy(ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    n, npx = 40, 3000
    cov = rng.random((n, npx)).astype(np.float32)
    cov[rng.random((n, npx)) < 0.5] = 0.0
    cov[3, :100] = 1.0
    a = rng.uniform(0.25, 1.0, n).astype(np.float32)
    a[3] = 1.0  # an opaque layer: its factor is 0 where it covers fully
    clr = np.concatenate([rng.random((n, 3)).astype(np.float32) * a[:, None], a[:, None]], axis=1)
    init = rng.random((npx, 4)).astype(np.float32)
    g_out = rng.standard_normal((npx, 4)).astype(np.float32)
    dev = torch.device("cuda")
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    out = torch.empty((npx, 4), dtype=torch.float32, device=dev)
    srcover_forward(ctx, t(cov.ravel()), n, npx, t(clr), out, init=t(init))
    gcov = torch.empty(n * npx, dtype=torch.float32, device=dev)
    ginit = torch.empty((npx, 4), dtype=torch.float32, device=dev)
    srcover_backward(ctx, t(cov.ravel()), n, npx, t(clr), t(g_out), gcov, init=t(init), grad_init=ginit)
    ctx.sync()
    # float64 reference by explicit stored states
    C = [init.astype(np.float64)]
    for i in range(n):
        C.append(clr[i][None, :] * cov[i][:, None] + C[-1] * (1 - clr[i][3] * cov[i])[:, None])
    assert np.abs(out.cpu().numpy() - C[-1]).max() < 1e-5
    G = g_out.astype(np.float64)
    want = np.zeros((n, npx))
    for i in reversed(range(n)):
        want[i] = (G * (clr[i][None, :] - clr[i][3] * C[i])).sum(axis=1)
        G = G * (1 - clr[i][3] * cov[i])[:, None]
    assert np.abs(gcov.cpu().numpy().reshape(n, npx) - want).max() < 1e-4 * np.abs(want).max()
    assert np.abs(ginit.cpu().numpy() - G).max() < 1e-5


@pytest.mark.parametrize("chunk", [0, 1, 3, 4])
def test_stroke_composite_matches_fp64_chain(ctx, chunk):
    torch = pytest.importorskip("torch")
    side = 96
    paths_ops, widths, clrs, _ = workloads.strokes_16384(n_paths=10, side=side, min_seg=3, max_seg=10)
    ops, paths, _ = pack_coverage(paths_ops, [side] * len(paths_ops))
    clr = clrs.astype(np.float64) / 255.0
    target = np.random.default_rng(9).random((side * side, 4))
    ctx.set_join(_abi.JOIN_MITER, 4.0)
    dev = torch.device("cuda")
    ops_d = torch.from_numpy(ops.view(np.uint8).copy()).to(dev)
    clr_d = torch.from_numpy(clr.astype(np.float32)).to(dev)
    tgt_d = torch.from_numpy(target.astype(np.float32)).to(dev)
    torch.cuda.synchronize()
    loss, out, g_ops, g_w, ms = stroke_composite_grads(ctx, ops_d, paths, clr_d, side, side, tgt_d, chunk=chunk)
    assert ms["chunk"] == (chunk or len(paths))
    loss64, C64, g64, gw64 = oracle.adj_stroke_composite(ops, paths, clr, side, side, target)
    assert np.abs(out.cpu().numpy() - C64).max() < 1e-4
    assert abs(float(loss) - loss64) <= 1e-4 * loss64
    scale = max(np.abs(g64).max(), np.abs(gw64).max())
    assert np.abs(g_ops.cpu().numpy() - g64).max() / scale < 2e-4
    assert np.abs(g_w.cpu().numpy() - gw64).max() / scale < 2e-4


def composite_case(n=9, side=80, seed=9):
    paths_ops, widths, clrs, _ = workloads.strokes_16384(n_paths=n, side=side, min_seg=3, max_seg=9)
    ops, paths, _ = pack_coverage(paths_ops, [side] * n)
    rng = np.random.default_rng(seed)
    return ops, paths, clrs.astype(np.float64) / 255.0, rng.random((side * side, 4)), rng.random((side * side, 4)) * 0.6


def test_host_buffers_initial_canvas_and_reuse(ctx):
    side = 80
    ops, paths, clr, target, init = composite_case(side=side)
    ctx.set_join(_abi.JOIN_MITER, 4.0)
    loss64, C64, g64, gw64, g0_64 = oracle.adj_stroke_composite(ops, paths, clr, side, side, target, init=init)
    comp = StrokeComposite(ctx)
    for _ in range(2):  # the saved state is reused; every backward recomputes what it needs
        out = np.zeros((side * side, 4), np.float32)
        comp.forward(ops, paths, clr.astype(np.float32), side, side, out, init=init.astype(np.float32), chunk=2)
        assert comp.chunk == 2 and (comp.status() == _abi.OK).all()
        assert np.abs(out - C64).max() < 1e-4
        g_out = (2.0 * (out.astype(np.float64) - target)).astype(np.float32)
        for _ in range(2):
            g_ops = np.full((len(ops), 6), 9.0, np.float32)
            g_w = np.full(len(paths), 9.0, np.float32)
            g0 = np.zeros((side * side, 4), np.float32)
            comp.backward(g_out, g_ops, g_w, g0)
            scale = max(np.abs(g64).max(), np.abs(gw64).max())
            assert np.abs(g_ops - g64).max() / scale < 2e-4
            assert np.abs(g_w - gw64).max() / scale < 2e-4
            assert np.abs(g0 - g0_64).max() < 2e-4 * np.abs(g0_64).max()
    comp.close()


def test_chunking_is_exact_reassociation(ctx):
    # the chunked canvas is the same SrcOver arithmetic as one pass (the coverage itself
    # sums cell areas with shared-memory atomics in any order); gradients agree to rounding
    torch = pytest.importorskip("torch")
    side = 72
    ops, paths, clr, target, _ = composite_case(n=12, side=side, seed=3)
    dev = torch.device("cuda")
    ops_d = torch.from_numpy(ops.view(np.uint8).copy()).to(dev)
    clr_d = torch.from_numpy(clr.astype(np.float32)).to(dev)
    tgt_d = torch.from_numpy(target.astype(np.float32)).to(dev)
    ctx.set_join(_abi.JOIN_MITER, 4.0)
    res = {k: stroke_composite_grads(ctx, ops_d, paths, clr_d, side, side, tgt_d, chunk=k) for k in (12, 5, 1)}
    ref = res[12]
    for k in (5, 1):
        assert (res[k][1] - ref[1]).abs().max().item() <= 1e-6
        scale = ref[2].abs().max().item()
        assert (res[k][2] - ref[2]).abs().max().item() <= 1e-5 * scale
        assert (res[k][3] - ref[3]).abs().max().item() <= 1e-5 * scale


def test_composite_bad_arguments(ctx):
    ops, paths, clr, target, _ = composite_case(n=2, side=32)
    comp = StrokeComposite(ctx)
    out = np.zeros((32 * 32, 4), np.float32)
    with pytest.raises(FootileError):
        comp.backward(out, np.zeros((len(ops), 6), np.float32))  # no forward yet
    with pytest.raises(FootileError):
        comp.forward(ops, paths, clr.astype(np.float32), 0, 32, out)  # empty canvas
    bad = paths.copy()
    bad[1]["n_ops"] = len(ops)
    with pytest.raises(FootileError):
        comp.forward(ops, bad, clr.astype(np.float32), 32, 32, out)  # ops out of range
    comp.close()
