"""The oracle against the golden fixtures generated from the reference's own
code and data (tests/golden/make_golden.py): bit-for-bit equality."""
import numpy as np
import pytest

from tests.conftest import golden

EVOLVE = ["ref_axion_rkn4", "ref_axion_rkn5", "ref_minimal_ssprk3", "ref_axion_leapfrog"]


@pytest.mark.parametrize("name", EVOLVE)
def test_evolve_golden(oracle, name):
    g = golden(name)
    out = oracle.evolve_periodic(str(g["project"]), int(g["integrator"]), g["state_in"],
                                 t0=float(g["t0"]), dt=float(g["dt"]), dx=float(g["dx"]),
                                 nsteps=int(g["nsteps"]), nghost=int(g["nghost"]))
    assert np.array_equal(out, g["state_out"])


def test_fopt_gw_golden(oracle):
    g = golden("ref_fopt_gw_leapfrog")
    out = oracle.evolve_periodic("FirstOrderPhaseTransition", 11, g["state_in"], t0=0.0,
                                 dt=float(g["dt"]), dx=float(g["dx"]), nsteps=int(g["nsteps"]),
                                 nghost=2, params=g["params"], gw_params=g["gw_params"],
                                 with_gw=True)
    assert np.array_equal(out, g["state_out"])


def test_rhs_golden(oracle):
    g = golden("ref_rhs")
    t, dt, dx = float(g["time"]), float(g["dt"]), float(g["dx"])
    assert np.array_equal(oracle.fill_rhs("AxionStrings", g["state16"], t, 0, dt, dx,
                                          with_gw=True, nghost=3), g["rhs_axion_gw"])
    ko = [0.1, 0.2, 0.3, 0.4]
    assert np.array_equal(oracle.fill_rhs("MinimalExample", g["state4"], t, 0, dt, dx, nghost=3,
                                          ko_order=2, ko_strength=ko), g["rhs_ko2"])
    assert np.array_equal(oracle.fill_rhs("MinimalExample", g["state4"], t, 0, dt, dx, nghost=3,
                                          ko_order=3, ko_strength=ko), g["rhs_ko3"])


def test_tag_golden(oracle):
    g = golden("ref_tag")
    m, c = oracle.tag("AxionStrings", g["state"], g["te"], 1.0, 0, float(g["dt"]),
                      float(g["dx"]), te_crit=g["te_crit"], max_grid=8)
    assert np.array_equal(m, g["mask"]) and np.array_equal(c, g["counts"])
    m0, c0 = oracle.tag("AxionStrings", g["state"], None, 1.0, 0, float(g["dt"]), float(g["dx"]),
                        max_grid=8)
    assert np.array_equal(m0, g["mask_user"]) and np.array_equal(c0, g["counts_user"])


def test_avgdown_te_golden(oracle):
    g = golden("ref_avgdown_te")
    c, t = oracle.avgdown_te(g["fine"], g["crse_in"], np.zeros_like(g["fine"]))
    assert np.array_equal(c, g["crse_out"]) and np.array_equal(t, g["te_out"])


@pytest.mark.parametrize("N", [32, 64])
def test_spectrum_bins_golden(oracle, N):
    g = golden(f"spectra_ks_{N}")
    assert np.array_equal(oracle.unique_k2(N), g["bins"])
    assert np.array_equal(oracle.index_to_k(N, 1), g["k1"])
    assert np.array_equal(oracle.index_to_k(N, 2), g["k2"])
