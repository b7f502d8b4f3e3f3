"""Coverage adjoint on the GPU against the FP64 gradient oracle.

The CUDA forward (FP32 analytic coverage) and backward (gradient of the loss with
respect to every op float, edges recomputed) go through the C ABI
(`ft_adjoint_forward` / `ft_adjoint_backward`) and are compared with the FP64
oracle on the same paths: coverage within 1e-4 absolute, gradients within 1e-4 of
the oracle's largest gradient entry (max |g - g64| / max |g64|) for NonZero.  Both
cover the same polygon (footile's f32 flattened vertices).  EvenOdd has a kink at
every integer winding area, NonZero at the clamp's 0 and 1; an edge pixel whose net
area lies within float rounding of a kink can take the other side of it in float
(in the self-intersecting mixed paths below one pixel has a net area of 2e-7 in
FP64 and clamps to 0 in float), so EvenOdd and the mixed paths are held to 5e-4."""
import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, workloads
from footile_gb300._lib import FootileError
from footile_gb300.adjoint import Adjoint, pack_coverage
from footile_gb300.path import Path2D

pytestmark = pytest.mark.gpu

COV_TOL = 1e-4
GRAD_TOL = {_abi.NONZERO: 1e-4, _abi.EVENODD: 5e-4}
KINK_TOL = 5e-4  # self-intersecting paths with pixels at a kink to float rounding


def run_gpu(ctx, rule, ops, paths, cov_bytes, target):
    adj = Adjoint(ctx)
    cov = np.zeros(cov_bytes // 4, np.float32)
    adj.forward(rule, ops, paths, cov)
    g_cov = (2.0 * (cov.astype(np.float64) - target)).astype(np.float32)
    g_ops = np.zeros((len(ops), 6), np.float32)
    adj.backward(g_cov, g_ops)
    st = adj.status()
    adj.close()
    return cov, g_cov, g_ops, st


def run_oracle(rule, ops, paths, g_cov, transform=_abi.IDENTITY, tolerance=0.3):
    covs, grads, sts = [], np.zeros((len(ops), 6)), []
    for p in paths:
        b, n, w, h = int(p["op_begin"]), int(p["n_ops"]), int(p["width"]), int(p["height"])
        o = ops[b:b + n]
        cov, area, st = oracle.adj_forward(rule, o, w, h, transform=transform, tolerance=tolerance)
        off = int(p["raster_offset"]) // 4
        gc = g_cov[off:off + w * h].reshape(h, w).astype(np.float64)
        grads[b:b + n] += oracle.adj_backward(rule, o, w, h, area, gc, transform=transform, tolerance=tolerance)
        covs.append(cov.ravel())
        sts.append(st)
    return np.concatenate(covs) if covs else np.zeros(0), grads, np.array(sts)


def check(ctx, rule, ops, paths, cov_bytes, seed=5, transform=_abi.IDENTITY, tolerance=0.3, grad_tol=None):
    target = np.random.default_rng(seed).random(cov_bytes // 4)
    cov, g_cov, g_ops, st = run_gpu(ctx, rule, ops, paths, cov_bytes, target)
    want_cov, want_g, want_st = run_oracle(rule, ops, paths, g_cov, transform, tolerance)
    assert (st == want_st).all(), (st, want_st)
    assert np.abs(cov - want_cov).max() < COV_TOL
    scale = np.abs(want_g).max()
    if scale > 0:
        err = np.abs(g_ops - want_g).max() / scale
        assert err < (grad_tol or GRAD_TOL[rule]), err
    else:
        assert not g_ops.any()
    return cov, g_ops


@pytest.mark.parametrize("rule", [_abi.NONZERO, _abi.EVENODD])
def test_cubic_batch_matches_fp64_oracle(ctx, rule):
    ops, paths, cov_bytes, _ = workloads.cubics_1024_coverage(n_paths=48)
    check(ctx, rule, ops, paths, cov_bytes)


def mixed_paths(seed, n):
    rng = np.random.default_rng(seed)
    per, sizes = [], []
    for i in range(n):
        side = int(rng.integers(8, 200))
        o = workloads.random_path(rng, side, int(rng.integers(1, 40)), n_sub=int(rng.integers(1, 4)),
                                  close=bool(i % 3))
        # some paths reach outside the raster on every side
        if i % 4 == 1:
            o["v"] = o["v"] * 1.6 - side * 0.3
        per.append(o)
        sizes.append((side, int(rng.integers(8, 200))) if i % 5 == 2 else side)
    return pack_coverage(per, sizes)


@pytest.mark.parametrize("rule", [_abi.NONZERO, _abi.EVENODD])
def test_mixed_paths_match_fp64_oracle(ctx, rule):
    ops, paths, cov_bytes = mixed_paths(21 + rule, 40)
    check(ctx, rule, ops, paths, cov_bytes, grad_tol=KINK_TOL)


def test_transform_and_tolerance(ctx):
    m = (0.8, 0.25, 6.0, -0.2, 1.15, -4.0)
    ops, paths, cov_bytes, _ = workloads.cubics_1024_coverage(n_paths=12)
    ctx.set_transform(m)
    ctx.set_tolerance(0.1)
    check(ctx, _abi.NONZERO, ops, paths, cov_bytes, transform=m, tolerance=0.1)


def test_example_shapes(ctx):
    fish = (Path2D().relative().move_to(112.0, 24.0).line_to(-32.0, 24.0).cubic_to(-96.0, -48.0, -96.0, 80.0, 0.0, 32.0)
            .line_to(32.0, 24.0).line_to(-16.0, -40.0).close().finish())
    heptagram = (Path2D().absolute().move_to(50, 0).line_to(89, 78).line_to(10, 31).line_to(90, 31).line_to(11, 78)
                 .close().finish())
    quads = (Path2D().absolute().move_to(10, 10).quad_to(60, -20, 90, 40).quad_to(40, 90, 5, 60).close().finish())
    empty = Path2D().absolute().move_to(3, 3).finish()
    ops, paths, cov_bytes = pack_coverage([fish, heptagram, quads, empty], [128, 100, (96, 80), 16])
    for rule in (_abi.NONZERO, _abi.EVENODD):
        check(ctx, rule, ops, paths, cov_bytes)


def test_wide_canvas_uses_several_bands(ctx):
    # 3000 x 40 floats exceed one 64 KB band: rows are covered band after band
    o = Path2D().absolute().move_to(-20, 5).cubic_to(1000, -30, 2000, 80, 3100, 20).line_to(2900, 39.5).close().finish()
    ops, paths, cov_bytes = pack_coverage([o], [(3000, 40)])
    check(ctx, _abi.NONZERO, ops, paths, cov_bytes)


def test_vertex_cap(ctx):
    n = 70000
    o = np.zeros(n + 2, dtype=_abi.OP_DTYPE)
    o["kind"][0] = _abi.OP_MOVE
    o["kind"][1:-1] = _abi.OP_LINE
    o["v"][:-1, :2] = np.random.default_rng(1).random((n + 1, 2)) * 50
    o["kind"][-1] = _abi.OP_CLOSE
    ok = Path2D().absolute().move_to(5, 5).line_to(40, 10).line_to(20, 40).close().finish()
    ops, paths, cov_bytes = pack_coverage([o, ok], [64, 64])
    target = np.zeros(cov_bytes // 4)
    cov, g_cov, g_ops, st = run_gpu(ctx, _abi.NONZERO, ops, paths, cov_bytes, target)
    assert st[0] == _abi.ERR_CAP and st[1] == _abi.OK
    assert not cov[:64 * 64].any() and cov[64 * 64:].any()
    assert not g_ops[:n + 2].any() and g_ops[n + 2:].any()


def test_device_buffers_and_reuse(ctx):
    torch = pytest.importorskip("torch")
    ops, paths, cov_bytes, target = workloads.cubics_1024_coverage(n_paths=16)
    host_cov, host_g = check(ctx, _abi.NONZERO, ops, paths, cov_bytes, seed=5)
    dev = torch.device("cuda")
    ops_d = torch.from_numpy(ops.view(np.uint8).copy()).to(dev)
    cov_d = torch.zeros(cov_bytes // 4, dtype=torch.float32, device=dev)
    adj = Adjoint(ctx)
    for _ in range(2):  # the saved state is reused by the second forward
        adj.forward(_abi.NONZERO, ops_d, paths, cov_d)
        # shared-memory float atomics sum the cell areas in any order
        assert np.abs(cov_d.cpu().numpy() - host_cov).max() < 1e-6
    tgt = np.random.default_rng(5).random(cov_bytes // 4)
    g_cov = torch.from_numpy((2.0 * (host_cov.astype(np.float64) - tgt)).astype(np.float32)).to(dev)
    g_ops = torch.empty((len(ops), 6), dtype=torch.float32, device=dev)
    g_w = torch.full((len(paths),), 7.0, device=dev)
    adj.backward(g_cov, g_ops, g_w)
    assert np.abs(g_ops.cpu().numpy() - host_g).max() <= 1e-5 * np.abs(host_g).max()
    assert not g_w.cpu().numpy().any()
    adj.close()


def test_torch_autograd_function(ctx):
    torch = pytest.importorskip("torch")
    from footile_gb300.adjoint import make_coverage_fn
    ops, paths, cov_bytes, target = workloads.cubics_1024_coverage(n_paths=8)
    dev = torch.device("cuda")
    ctrl = torch.tensor(np.array(ops["v"]), dtype=torch.float32, device=dev, requires_grad=True)
    tgt = torch.from_numpy(target).to(dev)
    fn = make_coverage_fn()
    adj = Adjoint(ctx)
    cov = fn.apply(ctrl, ops["kind"], paths, cov_bytes // 4, _abi.NONZERO, adj)
    loss = ((cov - tgt) ** 2).sum()
    loss.backward()
    ctx.sync()
    g = ctrl.grad.cpu().numpy()
    _, want_g, _ = run_oracle(_abi.NONZERO, ops, paths, (2 * (cov.detach().cpu().numpy() - target)).astype(np.float32))
    assert np.abs(g - want_g).max() / np.abs(want_g).max() < GRAD_TOL[_abi.NONZERO]
    adj.close()


def test_bad_arguments(ctx):
    ops, paths, cov_bytes, _ = workloads.cubics_1024_coverage(n_paths=2)
    adj = Adjoint(ctx)
    cov = np.zeros(cov_bytes // 4, np.float32)
    with pytest.raises(FootileError):
        adj.forward(_abi.NONZERO, ops, paths, cov[:-1])  # coverage outside the buffer
    bad = paths.copy()
    bad[0]["stride"] = 6
    with pytest.raises(FootileError):
        adj.forward(_abi.NONZERO, ops, bad, cov)
    with pytest.raises(FootileError):
        adj.backward(cov, np.zeros((len(ops), 6), np.float32))  # no successful forward yet
    adj.close()
