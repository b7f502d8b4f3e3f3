"""The oracle against every known-answer test footile holds for this path.

footile's own tests (Rust #[test]s) pin Fixed arithmetic (src/fixed.rs:166-313),
the figure rasteriser from fixed vertices to Matte8 / Rgba8p bytes
(src/fig.rs:691-794) and the row resolve (src/imgbuf.rs:205-232).  Each is
restated here with the same inputs and expected values.  CPU only.
"""
import math

import numpy as np
import pytest

import oracle
from footile_gb300 import _abi
from footile_gb300.path import Path2D, PathOp, ops_array

F = oracle.fx
ADD, SUB, MUL, DIV, SHL, SHR, ABS, FLOOR, CEIL, ROUND, TRUNC, FRACT, AVG = range(13)


def op(o, a, b=0):
    return oracle.fx_op(o, F(a) if not isinstance(a, np.int32) else a, F(b) if not isinstance(b, int) else b)


# ---------------------------------------------------------------- fixed.rs:166-313
def test_fixed_add():  # fixed.rs:166-174
    assert oracle.fx_op(ADD, F(1), F(1)) == F(2)
    assert oracle.fx_op(ADD, F(2), F(2)) == F(4)
    assert oracle.fx_op(ADD, F(2), F(-2)) == F(0)
    assert oracle.fx_op(ADD, F(2), F(-4)) == F(-2)
    assert oracle.fx_op(ADD, F(1.5), F(1.5)) == F(3)
    assert oracle.fx_op(ADD, F(3.5), F(-1.25)) == F(2.25)


def test_fixed_sub():  # fixed.rs:176-184
    assert oracle.fx_op(SUB, F(1), F(1)) == F(0)
    assert oracle.fx_op(SUB, F(3), F(2)) == F(1)
    assert oracle.fx_op(SUB, F(2), F(-2)) == F(4)
    assert oracle.fx_op(SUB, F(2), F(4)) == F(-2)
    assert oracle.fx_op(SUB, F(1.5), F(1.5)) == F(0)
    assert oracle.fx_op(SUB, F(3.5), F(1.25)) == F(2.25)


def test_fixed_mul():  # fixed.rs:186-194
    assert oracle.fx_op(MUL, F(2), F(2)) == F(4)
    assert oracle.fx_op(MUL, F(3), F(-2)) == F(-6)
    assert oracle.fx_op(MUL, F(4), F(0.5)) == F(2)
    assert oracle.fx_op(MUL, F(-16), F(-16)) == F(256)
    assert oracle.fx_op(MUL, F(37), F(3)) == F(111)
    assert oracle.fx_op(MUL, F(128), F(128)) == F(16384)


def test_fixed_div():  # fixed.rs:196-205
    assert oracle.fx_op(DIV, F(4), F(2)) == F(2)
    assert oracle.fx_op(DIV, F(-6), F(2)) == F(-3)
    assert oracle.fx_op(DIV, F(2), F(0.5)) == F(4)
    assert oracle.fx_op(DIV, F(256), F(-16)) == F(-16)
    assert oracle.fx_op(DIV, F(111), F(3)) == F(37)
    assert oracle.fx_op(DIV, F(37), F(3)) == F(12.33333)
    assert oracle.fx_op(DIV, F(16384), F(128)) == F(128)


def test_fixed_shl():  # fixed.rs:207-214
    assert oracle.fx_op(SHL, F(0), 2) == F(0)
    assert oracle.fx_op(SHL, F(1), 1) == F(2)
    assert oracle.fx_op(SHL, F(0.5), 1) == F(1)
    assert oracle.fx_op(SHL, F(0.25), 2) == F(1)
    assert oracle.fx_op(SHL, F(0.125), 3) == F(1)


def test_fixed_shr():  # fixed.rs:216-223
    assert oracle.fx_op(SHR, F(0), 2) == F(0)
    assert oracle.fx_op(SHR, F(1), 1) == F(0.5)
    assert oracle.fx_op(SHR, F(2), 1) == F(1)
    assert oracle.fx_op(SHR, F(4), 2) == F(1)
    assert oracle.fx_op(SHR, F(8), 3) == F(1)


@pytest.mark.parametrize("a,want", [(1, 1), (500, 500), (-500, 500), (-1.5, 1.5), (-2.5, 2.5)])
def test_fixed_abs(a, want):  # fixed.rs:225-232
    assert oracle.fx_op(ABS, F(a)) == F(want)


@pytest.mark.parametrize("a,want", [(1, 1), (500, 500), (1.5, 1), (1.99999, 1), (-0.0001, -1), (-2.5, -3)])
def test_fixed_floor(a, want):  # fixed.rs:234-242
    assert oracle.fx_op(FLOOR, F(a)) == F(want)


@pytest.mark.parametrize("a,want", [(1, 1), (500, 500), (1.5, 2), (1.99999, 2), (-0.0001, 0), (-2.5, -2)])
def test_fixed_ceil(a, want):  # fixed.rs:244-252
    assert oracle.fx_op(CEIL, F(a)) == F(want)


@pytest.mark.parametrize("a,want", [(1, 1), (500, 500), (1.5, 2), (1.49999, 1), (1.99999, 2), (-0.0001, 0),
                                    (-2.5, -2), (-2.9, -3)])
def test_fixed_round(a, want):  # fixed.rs:254-264
    assert oracle.fx_op(ROUND, F(a)) == F(want)


@pytest.mark.parametrize("a,want", [(1, 1), (500, 500), (1.5, 1), (1.49999, 1), (1.99999, 1), (-0.0001, 0),
                                    (-2.5, -2), (-2.9, -2)])
def test_fixed_trunc(a, want):  # fixed.rs:266-276
    assert oracle.fx_op(TRUNC, F(a)) == F(want)


@pytest.mark.parametrize("a,want", [(0, 0), (0.1, 0.1), (0.9, 0.9), (1.5, 0.5), (-2.5, 0.5)])
def test_fixed_fract(a, want):  # fixed.rs:278-285
    assert oracle.fx_op(FRACT, F(a)) == F(want)


def test_fixed_avg():  # fixed.rs:287-294
    assert oracle.fx_op(AVG, F(1), F(2)) == F(1.5)
    assert oracle.fx_op(AVG, F(1), F(1)) == F(1)
    assert oracle.fx_op(AVG, F(5), F(-5)) == F(0)
    assert oracle.fx_op(AVG, F(3), F(37)) == F(20)
    assert oracle.fx_op(AVG, F(3), F(1.5)) == F(2.25)


def test_fixed_into():  # fixed.rs:296-304
    assert oracle.fx_to_int(F(37)) == 37
    assert oracle.fx_to_f32(F(2.5)) == 2.5
    assert oracle.fx_to_int(F(2.5)) == 2


def test_fixed_cmp():  # fixed.rs:306-313
    assert F(37) > F(3)
    assert F(3) < F(37)
    assert F(-4) < F(4)
    assert min(F(37), F(3)) == F(3)
    assert max(F(37), F(3)) == F(37)


def test_fixed_from_f32_saturates():
    # Rust `as` casts saturate and send NaN to 0 (F10 of the figure path)
    assert F(40000.0) == 2**31 - 1
    assert F(-40000.0) == -(2**31)
    assert F(float("nan")) == 0


# ---------------------------------------------------------------------- fig.rs
def test_fixed_pt():  # fig.rs:691-700
    a = (F(2.0), F(1.0))
    b = (F(3.0), F(4.0))
    c = (F(-1.0), F(1.0))
    assert (oracle.fx_op(SUB, b[0], a[0]), oracle.fx_op(SUB, b[1], a[1])) == (F(1.0), F(3.0))
    assert oracle.widdershins(a, b)
    assert not oracle.widdershins(b, a)
    assert oracle.widdershins(b, c)


def fig_ops(points):
    """Fig::add_point for each point then close, expressed as Move + Lines."""
    return ops_array([PathOp.Move(*points[0])] + [PathOp.Line(*p) for p in points[1:]])


# (points, width, height, expected Matte8 bytes)  fig.rs:723-794
FIG_CASES = {
    "fig_9x1": ([(0.0, 0.0), (9.0, 1.0), (0.0, 1.0)], 9, 1, [242, 213, 185, 156, 128, 100, 71, 43, 14]),
    "fig_x_bounds": ([(-1.0, 0.0), (-1.0, 3.0), (3.0, 1.5)], 3, 3, [112, 16, 0, 255, 224, 32, 112, 16, 0]),
    "fig_partial": ([(0.5, 0.0), (0.5, 1.5), (1.0, 3.0), (1.0, 0.0)], 1, 3, [128, 117, 43]),
    "fig_partial2": ([(1.5, 0.0), (1.5, 1.5), (2.0, 3.0), (3.0, 3.0), (3.0, 0.0)], 3, 3,
                     [0, 128, 255, 0, 117, 255, 0, 43, 255]),
    "fig_partial3": ([(0.0, 0.0), (0.0, 0.3), (9.0, 0.0)], 9, 1, [73, 64, 56, 47, 39, 30, 22, 13, 4]),
}


@pytest.mark.parametrize("name", sorted(FIG_CASES))
def test_fig_matte8(name):
    pts, w, h, want = FIG_CASES[name]
    r = np.zeros((h, w), np.uint8)
    st, _ = oracle.fill(_abi.NONZERO, fig_ops(pts), r, _abi.MATTE8)
    assert st == 0
    assert r.ravel().tolist() == want


def test_fig_3x3_rgba8p():  # fig.rs:702-721
    r = np.zeros((3, 3, 4), np.uint8)
    oracle.fill(_abi.NONZERO, fig_ops([(1.0, 2.0), (1.0, 3.0), (2.0, 3.0), (2.0, 2.0)]), r, _abi.RGBA8P,
                (99, 99, 99, 255))
    want = np.zeros((3, 3, 4), np.uint8)
    want[2, 1] = (99, 99, 99, 255)
    assert np.array_equal(r, want)


# ------------------------------------------------------------------- imgbuf.rs
def test_imgbuf_non_zero():  # imgbuf.rs:205-221
    d, s = oracle.accumulate(_abi.NONZERO, [200] + [0] * 2999)
    assert (d == 200).all() and (s == 0).all()
    d, s = oracle.accumulate(_abi.NONZERO, [300] + [0] * 4999)
    assert (d == 255).all()


def test_imgbuf_even_odd():  # imgbuf.rs:223-232
    d, _ = oracle.accumulate(_abi.EVENODD, [300] + [0] * 2999)
    assert (d == 212).all()


# ------------------------------------------------------------------ plotter.rs
def test_plotter_overlapping_no_panic():  # plotter.rs:389-403 (asserts nothing but completion)
    path = (Path2D().absolute().move_to(8.0, 4.0).line_to(8.0, 3.0).cubic_to(8.0, 3.0, 8.0, 3.0, 9.0, 3.75)
            .line_to(8.0, 3.75).line_to(8.5, 3.75).line_to(8.5, 3.5).finish())
    r = np.zeros((16, 16), np.uint8)
    st, _ = oracle.fill(_abi.NONZERO, path, r, _abi.MATTE8)
    assert st == 0


def test_path2d_relative():  # path.rs:80-86, lib.rs:14-23 (the doc-test fish)
    fish = (Path2D().relative().pen_width(3.0).move_to(112.0, 24.0).line_to(-32.0, 24.0)
            .cubic_to(-96.0, -48.0, -96.0, 80.0, 0.0, 32.0).line_to(32.0, 24.0).line_to(-16.0, -40.0)
            .close().finish())
    assert fish["kind"].tolist() == [_abi.OP_PEN_WIDTH, _abi.OP_MOVE, _abi.OP_LINE, _abi.OP_CUBIC,
                                     _abi.OP_LINE, _abi.OP_LINE, _abi.OP_CLOSE]
    assert fish["v"][2, :2].tolist() == [80.0, 48.0]
    assert fish["v"][3].tolist() == [-16.0, 0.0, -16.0, 128.0, 80.0, 80.0]
    r = np.zeros((128, 128), np.uint8)
    st, sw = oracle.fill(_abi.NONZERO, fish, r, _abi.MATTE8)
    assert st == 0 and sw == 3.0 and r.max() == 255


# ----------------------------------------------------------- project-written math
def test_fmath_accuracy():
    rng = np.random.default_rng(0)
    for _ in range(2000):
        y, x = (rng.standard_normal(2) * 10 ** rng.uniform(-3, 3, 2)).astype(np.float32)
        a = oracle.atan2f(float(y), float(x))
        assert abs(a - math.atan2(float(y), float(x))) < 2e-6
    for v in np.linspace(-7, 7, 2001).astype(np.float32):
        assert abs(oracle.sinf(float(v)) - math.sin(float(v))) < 2e-6
    assert oracle.atan2f(0.0, -1.0) == pytest.approx(math.pi)
    assert oracle.atan2f(-0.0, -1.0) == pytest.approx(-math.pi)
