"""Scalar spectra and projections on the GPU against the oracle."""
import numpy as np
import pytest

import sledgehamr_gb300 as sh
from sledgehamr_gb300 import ic
from tests.amr_common import config, level0
from tests.oracle_lib import OracleAmr, oracle_out_function, oracle_scalar_spectrum

pytestmark = pytest.mark.gpu


def axion_state(N=16, seed=2):
    st = ic.axion_string_ic(N, 4.0, kmax=4.0, seed=seed)
    st[2:] = 0.3 * ic.axion_string_ic(N, 4.0, kmax=4.0, seed=seed + 1)[:2]
    return st


@pytest.mark.parametrize("fn,comp", [(0, 1), (1, 3), (2, 0), (3, 0), (4, 0)])
def test_scalar_spectrum_vs_oracle(ctx, fn, comp):
    N, dx, t = 16, 0.25, 1.3
    st = axion_state(N)
    lv = sh.Level.periodic(ctx, "AxionStringsLap1", N, 1, max_grid=8)
    lv.write(st)
    lv.set_time(t)
    bins, ks = lv.scalar_spectrum(fn, dx, comp)
    rb, rks = oracle_scalar_spectrum(st, fn, comp, N * dx, t)
    assert np.array_equal(ks, rks)
    scale = np.abs(rb).max()
    assert np.all(np.abs(bins - rb) <= 1e-10 * np.abs(rb) + 1e-14 * scale)
    lv.close()


@pytest.mark.parametrize("fn,mode", [(2, 0), (1, 1), (4, 0)])
def test_single_level_projection_bitwise(ctx, fn, mode):
    N = 16
    st = axion_state(N)
    lv = sh.Level.periodic(ctx, "AxionStringsLap1", N, 1, max_grid=8)
    lv.write(st)
    data, n = sh.projection(ctx, [lv], fn, comp=2, mode=mode)
    v = oracle_out_function(st, fn, 2)  # (z, y, x)
    if mode == 0:
        ref = np.cumsum(v, axis=0)[-1].T  # sequential sum over z, pixel [x, y]
    else:
        ref = np.maximum(0.0, v.max(axis=0)).T
    assert np.array_equal(data, ref)
    assert np.all(n == N)
    lv.close()


def test_amr_projection_vs_oracle(ctx):
    g = sh.Amr(ctx, config(), level0())
    o = OracleAmr(config(), level0())
    g.step(3)
    o.step(3)
    fin = g.info()["finest"]
    assert fin >= 1
    levels = [g.level(l) for l in range(fin + 1)]
    for fn, mode in ((2, 0), (3, 1)):
        data, n = sh.projection(ctx, levels, fn, comp=0, mode=mode)
        rd, rn = o.projection(fn, comp=0, mode=mode)
        assert np.array_equal(n, rn)
        assert np.max(np.abs(data - rd)) <= 1e-12 * max(np.abs(rd).max(), 1e-300)
    g.close()
    o.close()
