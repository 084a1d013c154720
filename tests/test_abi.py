"""The C ABI library loads, exports every symbol include/sledgehamr_gb300.h
declares, and its host-only entry points (project registry, spectrum bins,
index_to_k) agree with the reference's data.  No GPU is used."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import sledgehamr_gb300 as sh
from sledgehamr_gb300 import _lib
from tests.conftest import ROOT, golden


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from sledgehamr_gb300 import build
        build.build()
    return _lib.load()


def declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "sledgehamr_gb300.h")).read()
    return sorted(set(re.findall(r"^SH_API [^(]*?\b(sh_\w+)\(", hdr, flags=re.M)))


def test_every_declared_symbol_exported(lib):
    names = declared_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_project_registry(lib):
    assert lib.sh_project_count() == len(sh.PROJECTS)
    for q, name in enumerate(sh.PROJECTS):
        assert lib.sh_project_name(q).decode() == name
        assert sh.project_id(name) == q
    assert sh.project_ncomp("AxionStrings") == (4, 2)
    assert sh.project_ncomp("AxionStrings", True) == (16, 8)
    assert sh.project_ncomp("FirstOrderPhaseTransition", True) == (14, 7)
    with pytest.raises(sh.ShError):
        sh.project_ncomp("MinimalExample", True)
    with pytest.raises(sh.ShError):
        sh.project_id("NoSuchProject")


@pytest.mark.parametrize("N", [32, 64])
def test_spectrum_data_matches_reference_file(lib, N):
    g = golden(f"spectra_ks_{N}")
    assert np.array_equal(sh.spectrum_bins(N), g["bins"])
    for t in (1, 2):
        k = sh.index_to_k(N, t)
        ref = g[f"k{t}"]
        ulp = np.abs(k - ref) / np.spacing(np.maximum(np.abs(ref), 1e-300))
        assert ulp.max() <= 2


def test_spectrum_bins_large_against_oracle(lib, oracle):
    for N in (48, 96, 128):
        assert np.array_equal(sh.spectrum_bins(N), oracle.unique_k2(N))


def test_bad_arguments_rejected(lib):
    n = C.c_int()
    assert lib.sh_spectrum_bins(0, None, 0, C.byref(n)) == _lib.SH_ERR_ARG
    out = np.empty(8)
    assert lib.sh_index_to_k(8, 7, C.c_void_p(out.ctypes.data)) == _lib.SH_ERR_ARG
    assert lib.sh_ctx_create(0, None) == _lib.SH_ERR_ARG


def test_string_xi_restates_cosmology_xi():
    """sh_string_xi against Cosmology::Xi (projects/AxionStrings/
    cosmology.cpp:89-108, cosmology.h:77-97) written out here."""
    import math

    import sledgehamr_gb300 as sh
    T1, mpl, g = 5.4954174414835757e+17, 1.22e19, 106.0
    hub = math.sqrt(4.0 * math.pi ** 3 / 45.0 * g * T1 ** 4 / mpl ** 2)
    for tags, dx, L, eta in [(12345, 0.25, 64.0, 3.0), (1, 0.0625, 32.0, 0.5)]:
        length = tags * 2.0 / 3.0 * dx * eta / hub
        box = L * eta / hub
        t = 0.3012 / math.sqrt(g) * mpl / (T1 / eta) ** 2
        want = length * t ** 2 / box ** 3
        assert abs(sh.string_xi(tags, dx, L, eta) - want) <= 1e-14 * want
