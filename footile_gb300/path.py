"""`Path2D`, `PathOp`, `FillRule`, `JoinStyle` — the path-building side of footile.

Mirrors footile src/path.rs:8-171 and src/stroker.rs:13-20.  A built path is a
numpy array of `ft_op` records (32 bytes each), the input format of the C ABI.
Relative coordinates are resolved in f32 while building, as `Path2D::pt` does
(src/path.rs:80-86).
"""
import enum

import numpy as np

from . import _abi


class FillRule(enum.IntEnum):
    """src/path.rs:8-14"""
    NonZero = _abi.NONZERO
    EvenOdd = _abi.EVENODD


class JoinStyle:
    """src/stroker.rs:13-20: Miter(limit), Bevel, Round."""

    __slots__ = ("kind", "limit")

    def __init__(self, kind, limit=0.0):
        self.kind = int(kind)
        self.limit = float(limit)

    @classmethod
    def Miter(cls, limit):
        return cls(_abi.JOIN_MITER, limit)

    def __eq__(self, other):
        return isinstance(other, JoinStyle) and (self.kind, self.limit) == (other.kind, other.limit)

    def __repr__(self):
        if self.kind == _abi.JOIN_MITER:
            return f"JoinStyle.Miter({self.limit})"
        return "JoinStyle.Bevel" if self.kind == _abi.JOIN_BEVEL else "JoinStyle.Round"


JoinStyle.Bevel = JoinStyle(_abi.JOIN_BEVEL)
JoinStyle.Round = JoinStyle(_abi.JOIN_ROUND)


class PathOp:
    """src/path.rs:18-31.  Each constructor returns one `ft_op` record."""

    @staticmethod
    def _op(kind, *v):
        o = np.zeros((), dtype=_abi.OP_DTYPE)
        o["kind"] = kind
        o["v"][: len(v)] = np.asarray(v, dtype=np.float32)
        return o

    @staticmethod
    def Close():
        return PathOp._op(_abi.OP_CLOSE)

    @staticmethod
    def Move(x, y):
        return PathOp._op(_abi.OP_MOVE, x, y)

    @staticmethod
    def Line(x, y):
        return PathOp._op(_abi.OP_LINE, x, y)

    @staticmethod
    def Quad(bx, by, cx, cy):
        return PathOp._op(_abi.OP_QUAD, bx, by, cx, cy)

    @staticmethod
    def Cubic(bx, by, cx, cy, dx, dy):
        return PathOp._op(_abi.OP_CUBIC, bx, by, cx, cy, dx, dy)

    @staticmethod
    def PenWidth(w):
        return PathOp._op(_abi.OP_PEN_WIDTH, w)


def ops_array(ops):
    """Concatenate `ft_op` records (or arrays of them) into one contiguous array."""
    if isinstance(ops, np.ndarray) and ops.dtype == _abi.OP_DTYPE:
        return np.ascontiguousarray(ops.reshape(-1))
    parts = [np.asarray(o, dtype=_abi.OP_DTYPE).reshape(-1) for o in ops]
    if not parts:
        return np.zeros(0, dtype=_abi.OP_DTYPE)
    return np.ascontiguousarray(np.concatenate(parts))


class Path2D:
    """Builder for a vector of path ops (src/path.rs:44-171).  Relative by default."""

    def __init__(self):
        self._kinds = []
        self._vals = []
        self._absolute = False
        self._pen = (np.float32(0.0), np.float32(0.0))

    def absolute(self):
        self._absolute = True
        return self

    def relative(self):
        self._absolute = False
        return self

    def _pt(self, x, y):
        x = np.float32(x)
        y = np.float32(y)
        if self._absolute:
            return x, y
        return np.float32(self._pen[0] + x), np.float32(self._pen[1] + y)

    def _push(self, kind, vals):
        self._kinds.append(kind)
        self._vals.append(vals)

    def close(self):
        self._push(_abi.OP_CLOSE, ())
        self._pen = (np.float32(0.0), np.float32(0.0))
        return self

    def move_to(self, x, y):
        pb = self._pt(x, y)
        self._push(_abi.OP_MOVE, pb)
        self._pen = pb
        return self

    def line_to(self, x, y):
        pb = self._pt(x, y)
        self._push(_abi.OP_LINE, pb)
        self._pen = pb
        return self

    def quad_to(self, bx, by, cx, cy):
        pb = self._pt(bx, by)
        pc = self._pt(cx, cy)
        self._push(_abi.OP_QUAD, pb + pc)
        self._pen = pc
        return self

    def cubic_to(self, bx, by, cx, cy, dx, dy):
        pb = self._pt(bx, by)
        pc = self._pt(cx, cy)
        pd = self._pt(dx, dy)
        self._push(_abi.OP_CUBIC, pb + pc + pd)
        self._pen = pd
        return self

    def pen_width(self, width):
        self._push(_abi.OP_PEN_WIDTH, (np.float32(width),))
        return self

    def finish(self):
        ops = np.zeros(len(self._kinds), dtype=_abi.OP_DTYPE)
        for i, (k, v) in enumerate(zip(self._kinds, self._vals)):
            ops[i]["kind"] = k
            ops[i]["v"][: len(v)] = np.asarray(v, dtype=np.float32)
        return ops
