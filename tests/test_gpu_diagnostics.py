"""Diagnostics on device levels against the oracle / numpy, and the
non-finite check:
* Cosmology::GetStringTags (sh_level_string_tags) equals the number of
  user-tagged cells of the oracle's CPU tagger (the winding hook) on a
  periodic level, and sh_tag's user count on the levels of a hierarchy;
* NextToMinimalExample's <r> (SH_REDUCE_SUM_MODULUS) equals numpy's mean of
  sqrt(Psi1^2 + Psi2^2) within 1e-14;
* NaN and infinities written from the host are counted per component and
  reported as SH_ERR_NONFINITE, also by an AMR hierarchy that checks after
  every coarse step."""
import ctypes as C

import numpy as np
import pytest

import sledgehamr_gb300 as sh
from sledgehamr_gb300 import _lib, ic
from tests.amr_common import config, level0

pytestmark = pytest.mark.gpu


def test_string_tags_equal_oracle_user_tags(ctx, oracle):
    N, L = 32, 8.0
    st = ic.axion_string_ic(N, L, kmax=3.0, seed=7)
    lv = sh.Level.periodic(ctx, "AxionStrings", N, 2, max_grid=16)
    lv.write(st)
    lv.fill_patch()
    n = lv.string_tags(2.0, 0, 0.0625, 0.25)
    mask, counts = oracle.tag("AxionStrings", st, np.zeros_like(st), 2.0, 0, 0.0625, 0.25)
    assert n == int(mask.sum()) == int(counts[1]) > 0
    lv.close()


def test_string_tags_on_hierarchy_levels_equal_tag_counts(ctx):
    g = sh.Amr(ctx, config(), level0(2))
    g.step(3)
    assert g.info()["finest"] >= 1
    lib = _lib.load()
    for lev in range(g.info()["finest"] + 1):
        v = g.level(lev)
        t, _ = v.time()
        dx = 4.0 / (16 << lev)
        n = v.string_tags(t, lev, 0.25 * dx, dx)
        mask = np.empty(v.nvalid, dtype=np.uint8)
        counts = np.zeros(2 + v.ncomp, dtype=np.int64)
        ctx.check(lib.sh_tag(ctx.h, v.h, 0, t, lev, 0.25 * dx, dx, None, None, 0, None, 0,
                             C.c_void_p(mask.ctypes.data), C.c_void_p(counts.ctypes.data), None,
                             0, None), "sh_tag")
        assert n == counts[1] == mask.sum()
    g.close()


def test_mean_radial_mode_equals_numpy(ctx):
    N = 48
    st = ic.axion_string_ic(N, 12.0, kmax=2.0, seed=3)
    lv = sh.Level.periodic(ctx, "NextToMinimalExample", N, 2, max_grid=16)
    lv.write(st)
    want = float(np.mean(np.sqrt(st[0] ** 2 + st[1] ** 2)))
    assert abs(lv.mean_radial_mode(0) - want) <= 1e-14 * abs(want)
    lv.close()


def test_nonfinite_values_are_counted_and_reported(ctx):
    N = 24
    st = ic.axion_string_ic(N, 6.0, kmax=2.0, seed=5)
    lv = sh.Level.periodic(ctx, "AxionStrings", N, 2, max_grid=8)
    lv.write(st)
    assert lv.check_finite() == 0
    bad = st.copy()
    bad[1, 3, 4, 5] = np.nan
    bad[3, 0, 0, 0] = np.inf
    bad[3, 23, 23, 23] = -np.inf
    lv.write(bad)
    assert lv.reduce(sh.REDUCE_COUNT_NONFINITE, 1) == 1
    assert lv.reduce(sh.REDUCE_COUNT_NONFINITE, 3) == 2
    assert lv.reduce(sh.REDUCE_COUNT_NONFINITE, 0) == 0
    with pytest.raises(sh.ShError) as e:
        lv.check_finite()
    assert e.value.code == _lib.SH_ERR_NONFINITE
    assert "3 non-finite values" in str(e.value) and "component 1" in str(e.value)
    lv.close()


def test_amr_stops_on_nonfinite_state(ctx):
    g = sh.Amr(ctx, config(check_finite=1), level0(0))
    g.step(1)
    v = g.level(0)
    d = v.read()
    d[17] = np.nan
    v.write(d)
    with pytest.raises(sh.ShError) as e:
        g.step(1)
    assert e.value.code == _lib.SH_ERR_NONFINITE
    assert "level 0" in str(e.value)
    g.close()
