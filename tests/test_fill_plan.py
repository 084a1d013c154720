"""Fill planning (sledgehamr_gb300/csrc/sh_fill_plan.h), compiled for the
host: on periodic single-level and two-level layouts every cell a ghost
fill, a coarse link or a level-to-level fill must write is written by
exactly one rectangle, copies come from the valid cells of the named source
box through its periodic shift, interpolated cells are owned by no source
box and have their parents on the coarse level; overlapping boxes and an
uncovered coarse-fine region are rejected."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_fill_plans_cover_each_cell_once(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "fpc")
    r = subprocess.run([gxx, "-O2", "-std=c++17", "-fopenmp",
                        "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(ROOT, "sledgehamr_gb300", "csrc"),
                        os.path.join(HERE, "cpp", "fill_plan_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout
    assert out.stdout.strip().endswith("ok")
