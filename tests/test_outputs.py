"""Output functions, scalar spectra and projections (Spectrum::Compute,
Projection::Compute): the oracle against the reference's own per-cell
functions (bitwise) and against an independent numpy restatement."""
import numpy as np
import pytest

from sledgehamr_gb300 import ic
from tests.oracle_lib import (oracle_out_function, oracle_scalar_spectrum, ref_available)


def axion_state(N=12, seed=2):
    st = ic.axion_string_ic(N, 4.0, kmax=4.0, seed=seed)
    st[2:] = 0.3 * ic.axion_string_ic(N, 4.0, kmax=4.0, seed=seed + 1)[:2]
    return st


@pytest.mark.skipif(not ref_available(), reason="oracle/_ref not built")
@pytest.mark.parametrize("fn", [1, 2, 3, 4])
def test_out_functions_bitwise_vs_reference(fn):
    st = axion_state()
    comp = 1 if fn == 1 else 0
    a = oracle_out_function(st, fn, comp)
    b = oracle_out_function(st, fn, comp, ref=True)
    assert np.array_equal(a, b)


def test_scalar_spectrum_vs_numpy():
    N, L, t = 12, 4.0, 1.7
    st = axion_state(N)
    for fn, comp in ((0, 0), (1, 3), (2, 0), (4, 0)):
        bins, ks = oracle_scalar_spectrum(st, fn, comp, L, t)
        f = oracle_out_function(st, fn, comp)
        F = np.fft.rfftn(f)  # axes (z, y, x): x halved, as the R2C transform
        H = N // 2 + 1
        a = np.arange(H)[None, None, :]
        multpl = np.where((a == 0) | (a == N // 2), 1.0, 2.0)
        n = np.fft.fftfreq(N, 1.0 / N).astype(int)
        k2 = (n[:, None, None] ** 2 + n[None, :, None] ** 2 + np.arange(H)[None, None, :] ** 2)
        pre = t / N ** 6 / (2 * np.pi / L)
        ref = np.zeros(len(ks))
        idx = np.searchsorted(ks, k2.ravel())
        np.add.at(ref, idx, (multpl * np.abs(F) ** 2).ravel() * pre)
        scale = np.abs(ref).max()
        assert np.all(np.abs(bins - ref) <= 1e-12 * np.abs(ref) + 1e-14 * scale), fn
