"""Stroke points of the adjoint: the CTA-parallel walk (stroke_points_block in
ft_adjoint.cu) stores the same stroke points and sub-strokes, bit for bit, as a walk of
the ops one by one (Plotter's pen walk into Stroke::add_point / close, plotter.rs:175-332,
stroker.rs:204-236).  tests/cpp/stroke_points_check.cu runs both on seeded random paths
and exits non-zero on any difference."""
import os
import subprocess

import pytest

from footile_gb300 import _build

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_stroke_points_block_matches_one_thread(cuda_ok, tmp_path):
    exe = tmp_path / "stroke_points_check"
    flags = [f for f in _build.NVFLAGS if f not in ("-Xcompiler", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off")]
    flags += ["-Xcompiler", "-ffp-contract=off"]
    subprocess.check_call([_build.nvcc(), *flags, *_build.GENCODE, "-I",
                           os.path.join(ROOT, "footile_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "cpp", "stroke_points_check.cu"), "-o", str(exe)])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "mismatching paths 0" in out.stdout
    # the cap path and the several-window chunk were reached
    assert "max 65535 per path" in out.stdout
