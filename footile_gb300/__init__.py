"""footile_gb300 — GB300 (sm_103a) fill/stroke rasterisation path of footile."""
from ._abi import *  # noqa: F401,F403
from .path import FillRule, JoinStyle, Path2D, PathOp, ops_array  # noqa: F401
from .plotter import (Plotter, PreparedBatch, composite_batch, fill_batch, pack_batch,  # noqa: F401,E402
                      pen_width_chain, raster_format)
