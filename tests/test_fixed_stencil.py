"""The device Laplacian's integer ring sums and the device Gradient<2>,
<3> (include/sledgehamr/sh_fixed_stencil.h), compiled for the host: the
integer-only conversion of the sum equals the FP64 conversion bit for bit;
error
against the exact (binary128) value no larger than the FP64 evaluation's
(within 1.25 times it for the 19-point Laplacian), exact scaling by powers
of two, zeros, NaN and infinity."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_fixed_point_laplacian_host(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "fsc")
    r = subprocess.run([gxx, "-O2", "-std=gnu++17", "-I" + os.path.join(ROOT, "include", "sledgehamr"),
                        os.path.join(HERE, "cpp", "fixed_stencil_check.cpp"), "-o", exe,
                        "-lquadmath"], capture_output=True, text=True)
    if r.returncode != 0 and "quadmath" in (r.stderr + r.stdout):
        pytest.skip("libquadmath not available")
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout
    rows = [l.split() for l in out.stdout.strip().splitlines()]
    assert [r[0] for r in rows] == ["c", "1", "2", "3", "g2", "g3"]
    assert int(rows[0][1]) > 1000000  # integer-only conversions checked
    for order, fixed, fp64 in rows[1:]:
        assert float(fixed) <= float(fp64) * (1.25 if order == "3" else 1.0001) + 1.0
