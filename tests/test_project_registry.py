"""Projects register themselves (SH_DEFINE_PROJECT): a project written as a
header plus one .cu file (tests/cpp/wave_project.cu) and linked with the
library's objects, without any edit of the library, appears in the project
table after the built-in projects, whose ids (the oracle's numbering) do not
change.  Host only: the table is read through the C ABI without a GPU."""
import ctypes as C
import glob
import os
import shutil
import subprocess

import pytest

from tests.conftest import ROOT

PKG = os.path.join(ROOT, "sledgehamr_gb300")


def test_added_project_registers_itself(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    from sledgehamr_gb300 import build as pkg_build
    pkg_build.build()
    objs = [o for o in glob.glob(os.path.join(PKG, "_build", "*.o"))]
    assert objs
    obj = str(tmp_path / "wave_project.o")
    r = subprocess.run([nvcc] + pkg_build.ARCH + pkg_build.NVCC_FLAGS +
                       ["-I" + os.path.join(PKG, "csrc"), "-c",
                        os.path.join(ROOT, "tests", "cpp", "wave_project.cu"), "-o", obj],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    so = str(tmp_path / "libwithwave.so")
    r = subprocess.run([nvcc] + pkg_build.ARCH + ["-shared", "-o", so] + objs + [obj] +
                       ["-lcufft", "-lcudart", "-Xcompiler", "-fopenmp"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(so)
    lib.sh_project_find.restype = C.c_int
    lib.sh_project_count.restype = C.c_int
    lib.sh_project_ncomp.restype = C.c_int
    ids = {}
    for name in ("AxionStrings", "MinimalExample", "NextToMinimalExample",
                 "FirstOrderPhaseTransition", "AxionStringsLap1", "AxionStringsLap2",
                 "AxionStringsLap3", "WaveTest"):
        pid = C.c_int(-1)
        assert lib.sh_project_find(name.encode(), C.byref(pid)) == 0, name
        ids[name] = pid.value
    assert [ids[n] for n in list(ids)[:7]] == list(range(7))
    assert ids["WaveTest"] == 7 and lib.sh_project_count() == 8
    nc, npair = C.c_int(), C.c_int()
    assert lib.sh_project_ncomp(ids["WaveTest"], 0, C.byref(nc), C.byref(npair)) == 0
    assert (nc.value, npair.value) == (2, 1)
