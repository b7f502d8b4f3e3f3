"""The C++ host mirror (include/footile.hpp) drives the C ABI like footile's own
API: the fishy example (examples/fishy.rs) — a fill and two strokes on one
Rgba8p Plotter — must equal the oracle's sequence of the same Plotter calls."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from footile_gb300 import _abi, _build
from footile_gb300.path import Path2D

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_lib_dir():
    nvcc = _build.nvcc()
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "lib64")


@pytest.mark.parametrize("link", ["shared", "static"])
def test_cpp_mirror_fishy(cuda_ok, gpu_lib, tmp_path, link):
    exe = tmp_path / "fishy_demo"
    lib_dir = os.path.dirname(_build.LIB)
    src = [os.path.join(ROOT, "tests", "cpp", "fishy_demo.cpp")]
    if link == "shared":
        libs = ["-L", lib_dir, "-lfootile_gpu", f"-Wl,-rpath,{lib_dir}"]
    else:  # the static library, as a Rust crate's build.rs would link it
        libs = [_build.STATIC_LIB, "-L", _cuda_lib_dir(), "-lcudart_static", "-ldl", "-lpthread", "-lrt"]
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include")] + src +
                          ["-o", str(exe)] + libs)
    out = subprocess.run([str(exe), str(tmp_path / "rgba.bin"), str(tmp_path / "matte.bin")],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert "pen width 2.0" in out.stdout
    got_rgba = np.fromfile(tmp_path / "rgba.bin", np.uint8).reshape(128, 128, 4)
    got_matte = np.fromfile(tmp_path / "matte.bin", np.uint8).reshape(128, 128)

    fish = (Path2D().relative().pen_width(3.0).move_to(112.0, 24.0).line_to(-32.0, 24.0)
            .cubic_to(-96.0, -48.0, -96.0, 80.0, 0.0, 32.0).line_to(32.0, 24.0).line_to(-16.0, -40.0)
            .close().finish())
    eye = (Path2D().relative().pen_width(2.0).move_to(24.0, 48.0).line_to(8.0, 8.0).move_to(0.0, -8.0)
           .line_to(-8.0, 8.0).finish())
    want = np.zeros((128, 128, 4), np.uint8)
    _, sw = oracle.fill(_abi.NONZERO, fish, want, _abi.RGBA8P, (127, 96, 96, 255))
    _, sw = oracle.stroke(fish, want, _abi.RGBA8P, (255, 208, 208, 255), s_width=sw)
    _, sw = oracle.stroke(eye, want, _abi.RGBA8P, (0, 0, 0, 255), s_width=sw)
    assert sw == 2.0
    assert np.array_equal(got_rgba, want)
    want_m = np.zeros((128, 128), np.uint8)
    oracle.fill(_abi.NONZERO, fish, want_m, _abi.MATTE8)
    assert np.array_equal(got_matte, want_m)
