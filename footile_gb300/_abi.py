"""Plain-data layouts and constants of the C ABI declared in include/footile_gpu.h.

Pure Python + numpy: importing this module loads no native code.
"""
import numpy as np

# status codes
OK = 0
ERR_ARG = 1
ERR_DEPTH = 2
ERR_CAP = 3
ERR_TIMEOUT = 4
ERR_CUDA = 5
ERR_NOMEM = 6
STATUS_NAMES = {OK: "OK", ERR_ARG: "ERR_ARG", ERR_DEPTH: "ERR_DEPTH", ERR_CAP: "ERR_CAP",
                ERR_TIMEOUT: "ERR_TIMEOUT", ERR_CUDA: "ERR_CUDA", ERR_NOMEM: "ERR_NOMEM"}

MAX_DEPTH = 22
MAX_POINTS = 65535
MAX_WIDTH = 16384

# PathOp kinds (footile src/path.rs:18-31)
OP_CLOSE = 0
OP_MOVE = 1
OP_LINE = 2
OP_QUAD = 3
OP_CUBIC = 4
OP_PEN_WIDTH = 5

# FillRule (src/path.rs:8-14)
NONZERO = 0
EVENODD = 1

# JoinStyle (src/stroker.rs:13-20)
JOIN_MITER = 0
JOIN_BEVEL = 1
JOIN_ROUND = 2

# pixel formats
MATTE8 = 0
RGBA8P = 1
BYTES_PER_PIXEL = {MATTE8: 1, RGBA8P: 4}

HOST = 0
DEVICE = 1

# output formats of ft_convert (pix SRgba8 / SGray8)
SRGBA8 = 2
SGRAY8 = 3

# struct ft_op (32 bytes)
OP_DTYPE = np.dtype([("kind", "<i4"), ("v", "<f4", (6,)), ("reserved", "<i4")], align=True)
assert OP_DTYPE.itemsize == 32

# struct ft_path_desc (40 bytes)
PATH_DTYPE = np.dtype([
    ("op_begin", "<u4"), ("n_ops", "<u4"), ("width", "<u4"), ("height", "<u4"),
    ("raster_offset", "<u8"), ("stride", "<u4"), ("s_width", "<f4"),
    ("clr", "u1", (4,)), ("reserved", "<u4"),
], align=True)
assert PATH_DTYPE.itemsize == 40

IDENTITY = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0)
