"""The stroker's join decisions (footile src/stroker.rs:340-396) against libm.

footile decides a miter (`sm >= 1/ml && sm < 1`, sm = |sin(th/2)|) and a round join
(`th > 0`) from f32 `atan2` and `sin` of the platform libm.  The oracle and the CUDA
path share include/ft_fmath.h, which takes each decision as a correctly rounded f32
libm takes it.  These tests count, on the benchmark's stroke workloads, the joins whose
decision differs from the one taken with this machine's C library atan2f / sinf
(the functions Rust's f32::atan2 / f32::sin call), and check with 200-bit arithmetic
that at every such join ft_fmath.h's decision is the correctly rounded one — so each
remaining difference is the C library's own rounding."""
import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, workloads
from footile_gb300.path import PathOp, ops_array

mp = pytest.importorskip("mpmath")
mp.mp.prec = 200
F32 = np.float32


def rn32(x):
    """Round an mpmath value to the nearest f32 (ties to even), without double rounding."""
    f = F32(float(x))
    best = f
    for c in (np.nextafter(f, F32(-np.inf)), np.nextafter(f, F32(np.inf))):
        dc, db = abs(mp.mpf(float(c)) - x), abs(mp.mpf(float(best)) - x)
        if dc < db or (dc == db and (c.view(np.uint32) & 1) == 0):
            best = c
    return best


def fold(d):
    pi = F32(np.pi)
    if d < -pi:
        return F32(d + F32(2.0) * pi)
    if d > pi:
        return F32(d - F32(2.0) * pi)
    return d


def cr_decision(u, kind, ml=4.0):
    """The join decision with correctly rounded f32 atan2 and sin (200-bit arithmetic)."""
    ux, uy, vx, vy = (mp.mpf(float(F32(x))) for x in u)
    a = rn32(mp.atan2(uy, ux))
    b = rn32(mp.atan2(vy, vx))
    th = fold(F32(a - b))
    if kind == "round":
        return 2 if not (th <= 0) else 0
    sm_min = F32(F32(1.0) / F32(ml))
    sm = abs(rn32(mp.sin(mp.mpf(float(F32(th / F32(2.0)))))))
    return 1 if (sm >= sm_min and sm < F32(1.0)) else 0


def _flips(ops, kind, ml=4.0):
    join = _abi.JOIN_ROUND if kind == "round" else _abi.JOIN_MITER
    mine, uv = oracle.join_decisions(ops, join=join, miter_limit=ml, with_uv=True)
    libm = oracle.join_decisions(ops, libm=True, join=join, miter_limit=ml)
    assert len(mine) == len(libm)
    return mine, libm, uv, np.flatnonzero(mine != libm)


def test_sin_threshold_constant():
    # RN(sin x) < 1 exactly up to 1.570552110671997 (0x3FC907DA)
    f1 = F32(1.570552110671997)
    assert f1.view(np.uint32) == 0x3FC907DA
    assert rn32(mp.sin(mp.mpf(float(f1)))) < 1
    assert rn32(mp.sin(mp.mpf(float(np.nextafter(f1, F32(2)))))) == 1


def test_scene_stroke_round_joins():
    """The 4096x4096 scene stroked at width 8 with round joins (131,030 joins)."""
    ops, _, _, _ = workloads.scene_4096()
    sops = np.concatenate([ops_array([PathOp.PenWidth(8.0)]), ops])
    mine, libm, uv, flips = _flips(sops, "round")
    assert len(mine) > 100000
    for i in flips:
        assert mine[i] == cr_decision(uv[i], "round"), f"join {i}"
    assert len(flips) <= 10


def test_strokes_miter_joins():
    """The first 512 of the ordered composite's 16,384 strokes, Miter(4) (about 2.8 M
    joins; all 16,384 strokes: 88.7 M joins, 102 differ from this C library's)."""
    paths_ops, _, _, _ = workloads.strokes_16384()
    total, flips_all = 0, 0
    for o in paths_ops[:512]:
        mine, libm, uv, flips = _flips(o, "miter")
        total += len(mine)
        flips_all += len(flips)
        for i in flips:
            assert mine[i] == cr_decision(uv[i], "miter"), f"join {i}"
    assert total > 2000000
    assert flips_all <= 0.0001 * total


@pytest.mark.parametrize("ml", [1.0, 1.5, 4.0, 10.0, 1e30])
def test_near_threshold_joins_are_correctly_rounded(ml):
    """Random joins placed near every decision threshold (near-straight, near the miter
    limit, near a reversal), decided by ft_fmath.h as 200-bit arithmetic rounds them."""
    rng = np.random.default_rng(int(ml * 10) % 1000)
    sm_min = 1.0 / ml
    thetas = [np.pi - 2 * np.arcsin(1 - 2.0 ** -25), np.pi]
    if sm_min <= 1:
        thetas.append(2 * np.arcsin(sm_min))
    for k in range(300):
        t0 = thetas[k % len(thetas)] * (1 if k % 2 else -1) + rng.normal() * 3e-6
        phi = rng.uniform(-np.pi, np.pi)
        r1, r2 = rng.uniform(0.01, 50, 2)
        u = np.array([np.cos(phi) * r1, np.sin(phi) * r1], np.float32)
        w = np.array([np.cos(phi - t0) * r2, np.sin(phi - t0) * r2], np.float32)
        # a segment pair whose join has u = a1 - a0 and v = b0 - b1 = w
        ops = ops_array([PathOp.PenWidth(2.0), PathOp.Move(500.0, 500.0),
                         PathOp.Line(500.0 + float(u[0]), 500.0 + float(u[1])),
                         PathOp.Line(500.0 + float(u[0]) - float(w[0]), 500.0 + float(u[1]) - float(w[1]))])
        for kind in ("miter", "round"):
            join = _abi.JOIN_ROUND if kind == "round" else _abi.JOIN_MITER
            mine, uv = oracle.join_decisions(ops, join=join, miter_limit=ml, with_uv=True)
            for d, q in zip(mine, uv):
                want = cr_decision(q, kind, ml)
                assert d == want, (kind, ml, q, d, want)
