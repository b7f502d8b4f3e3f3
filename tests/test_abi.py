"""CPU checks of the C ABI: the library builds for sm_103a, loads, exports every
function include/footile_gpu.h declares, and its structs match the Python
layouts.  No compute call is made (no GPU here)."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np

from footile_gb300 import _abi, _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "footile_gpu.h")


def declared_functions():
    src = open(HEADER).read()
    return re.findall(r"FT_API\s+[\w\s\*]+?\b(ft_\w+)\s*\(", src)


def test_library_builds_and_exports_header_symbols():
    path = _build.build()
    lib = ctypes.CDLL(path)
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(_lib.exported_symbols()) | set(names)


def test_struct_layouts_match_c():
    src = f"""
#include <stdio.h>
#include <stddef.h>
#include "{HEADER}"
int main(void) {{
  printf("%zu %zu %zu %zu %zu\\n", sizeof(ft_op), sizeof(ft_path_desc), offsetof(ft_path_desc, raster_offset),
         offsetof(ft_path_desc, s_width), offsetof(ft_path_desc, clr));
  return 0;
}}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-o", exe, c])
        out = subprocess.check_output([exe]).decode().split()
    got = [int(v) for v in out]
    want = [_abi.OP_DTYPE.itemsize, _abi.PATH_DTYPE.itemsize, _abi.PATH_DTYPE.fields["raster_offset"][1],
            _abi.PATH_DTYPE.fields["s_width"][1], _abi.PATH_DTYPE.fields["clr"][1]]
    assert got == want


def test_header_constants_match_python():
    src = open(HEADER).read()
    for name, val in [("FT_MAX_DEPTH", _abi.MAX_DEPTH), ("FT_MAX_POINTS", _abi.MAX_POINTS),
                      ("FT_MAX_WIDTH", _abi.MAX_WIDTH)]:
        assert re.search(rf"#define {name} {val}\b", src), name
    for name, val in [("FT_OP_CUBIC", _abi.OP_CUBIC), ("FT_RGBA8P", _abi.RGBA8P), ("FT_JOIN_ROUND", _abi.JOIN_ROUND),
                      ("FT_ERR_DEPTH", _abi.ERR_DEPTH), ("FT_EVENODD", _abi.EVENODD)]:
        assert re.search(rf"{name} = {val}\b", src), name


def test_ctx_create_without_gpu_fails_cleanly():
    try:
        import torch
        if torch.cuda.is_available():
            return
    except Exception:
        pass
    L = _lib.load()
    h = ctypes.c_void_p()
    rc = L.ft_ctx_create(0, ctypes.byref(h))
    assert rc == _abi.ERR_CUDA and not h.value


def test_no_cpu_fallback_in_product():
    # the shipped package never imports the oracle
    pkg = os.path.join(ROOT, "footile_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                text = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in text and "oracle/" not in text, f


def test_ops_layout_roundtrip():
    from footile_gb300.path import Path2D
    ops = Path2D().absolute().move_to(1, 2).quad_to(3, 4, 5, 6).cubic_to(1, 2, 3, 4, 5, 6).close().finish()
    raw = ops.view(np.uint8).reshape(-1, 32)
    assert raw.shape == (4, 32)
    assert np.frombuffer(raw[1, :4].tobytes(), np.int32)[0] == _abi.OP_QUAD
    assert np.frombuffer(raw[2, 4:28].tobytes(), np.float32).tolist() == [1, 2, 3, 4, 5, 6]
