"""The numpy restatement of the GW spectrum (tests/gw_numpy.py), used by
the GPU parity tests on grids too large for the oracle's own transform,
equals the oracle's gw_spectrum on small grids: every bin within 1e-12
relative (summation order differs), the same bin list."""
import numpy as np
import pytest

from sledgehamr_gb300 import ic
from tests import gw_numpy


@pytest.mark.parametrize("N,zp", [(16, 1), (12, 2), (18, 1)])
@pytest.mark.parametrize("unbinned", [True, False])
def test_numpy_gw_spectrum_equals_oracle(oracle, N, zp, unbinned):
    comps = np.stack([ic.gaussian_field(N, 4.0, 8.0, 300 + q) for q in range(6)])
    want, wks = oracle.gw_spectrum(comps, zero_padding=zp, projection_type=2, unbinned=unbinned)
    got, ks = gw_numpy.gw_spectrum(comps, zp, 2, unbinned, oracle.index_to_k, oracle.unique_k2,
                                   chunk=5)
    assert np.array_equal(ks, wks)
    scale = np.abs(want).max()
    assert np.all(np.abs(got - want) <= 1e-12 * np.abs(want) + 1e-15 * scale)
