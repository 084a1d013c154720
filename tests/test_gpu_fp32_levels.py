"""FP32 + Kahan levels and AMR hierarchies (sh_level_create_prec,
csrc/sh_stage32.cuh): the precision form on the drop-in path, with FP32
values and compensations, FP32 stage arithmetic, FP32 ghost fills,
average-down sums as FP32 TwoSum pairs, and the truncation errors, tags
through the project's hooks and time in FP64.

* A periodic FP32 level, in one box or in several (ghost cells from the
  same-level copies), evolves bit for bit as the FP32 + Kahan ensemble
  kernels do on the same FP32-representable state: same stage schedule,
  same explicitly rounded FP32 arithmetic.
* Tags of an FP32 level (winding through the hooks on the FP64 values v - c)
  and its reductions equal those of an FP64 level holding the same values.
* An FP32 hierarchy against the FP64 oracle's hierarchy: the same levels and
  boxes after every coarse step, fields within 2e-6 relative L2 per level
  (the FP32 rounding of the stencils; 1e-7 to 4e-7 measured), regrid masks
  compared cell by cell with the mismatches counted (none measured).
* A checkpoint of an FP32 hierarchy restarts to the same evolution.
* FirstOrderPhaseTransition + GW on FP32 levels (leapfrog) against the FP32
  ensemble kernel and the FP64 oracle; bubbles on FP32 levels; an FP32
  hierarchy of that project against the FP64 oracle's.
* FP64-only operations refuse FP32 levels with SH_ERR_UNSUPPORTED.
"""
import numpy as np
import pytest

import sledgehamr_gb300 as sh
from sledgehamr_gb300 import _lib, ic
from tests.amr_common import config, level0
from tests.conftest import rel_l2
from tests.oracle_lib import OracleAmr

pytestmark = pytest.mark.gpu
F32 = sh.PREC_FP32_KAHAN


def _state(N, L, seed):
    """An axion-string state whose values are FP32 numbers (so an upload
    leaves zero compensations, as an ensemble upload does)."""
    st = ic.axion_string_ic(N, L, kmax=1.5, seed=seed)
    st[2:] = 0.2 * ic.axion_string_ic(N, L, kmax=1.0, seed=seed + 100)[:2]
    return st.astype(np.float32).astype(np.float64)


@pytest.mark.parametrize("order", [1, 2])
def test_fp32_level_equals_fp32_ensemble(ctx, order):
    N, dx, dt, t0, steps = 32, 0.25, 0.0625, 0.7, 6
    params = [0.8, 0.1]
    st = _state(N, N * dx, 3 + order)
    fam = sh.FAMILY_AXION_LAP1 if order == 1 else sh.FAMILY_AXION_LAP2
    E = sh.Ensemble(ctx, fam, F32, [N], [dx], params + [0.0, 0.0])
    E.write(0, st)
    E.set_time(t0)
    E.step(dt, steps)
    ref = np.asarray(E.read(0)).ravel()
    E.close()
    for max_grid in (0, 16):
        lv = sh.Level.periodic(ctx, f"AxionStringsLap{order}", N, order, max_grid=max_grid,
                               precision=F32)
        lv.write(st)
        lv.set_time(t0)
        for _ in range(steps):
            lv.advance(sh.RKN4, dt, dx, params=params)
        out = lv.read().ravel()
        assert abs(lv.time()[0] - (t0 + dt * steps)) < 1e-12
        lv.close()
        assert np.array_equal(out, ref), (max_grid, rel_l2(out, ref))


def test_fp32_level_tags_and_reductions_equal_fp64(ctx):
    N, L = 32, 8.0
    st = _state(N, L, 11)
    a = sh.Level.periodic(ctx, "AxionStringsLap2", N, 2, max_grid=16, precision=F32)
    b = sh.Level.periodic(ctx, "AxionStringsLap2", N, 2, max_grid=16)
    for lv in (a, b):
        lv.write(st)
        lv.fill_patch()
    ma, ca, _ = a.tag(1.0, 0, 0.0625, 0.25)
    mb, cb, _ = b.tag(1.0, 0, 0.0625, 0.25)
    assert ma.sum() > 0
    assert np.array_equal(ma, mb) and np.array_equal(ca, cb)
    for op in (sh.REDUCE_MAX_ABS, sh.REDUCE_SUM, sh.REDUCE_SUM_MODULUS):
        assert a.reduce(op, 0) == b.reduce(op, 0)
    assert a.string_tags(1.0, 0, 0.0625, 0.25) == b.string_tags(1.0, 0, 0.0625, 0.25)
    assert np.array_equal(a.read(), st)
    a.close()
    b.close()


def test_fp32_hierarchy_against_fp64_oracle(ctx):
    g = sh.Amr(ctx, config(precision=F32), level0())
    o = OracleAmr(config(), level0())
    errors = []
    for step in range(4):
        g.step(1)
        o.step(1)
        gi, oi = g.info(), o.info()
        assert gi["finest"] == oi["finest"], step
        assert gi["cell_updates"] == oi["cell_updates"]
        for lev in range(gi["finest"] + 1):
            assert g.level(lev).boxes == o.boxes(lev), (step, lev)
            e = rel_l2(g.level(lev).read(), o.read(lev)[0])
            errors.append((step, lev, e))
            assert e <= 2e-6, (step, lev, e)
    assert g.info()["finest"] >= 1
    mism, cells = 0, 0
    for q in range(g.info()["nregrids"]):
        rg, ro = g.regrid_record(q), o.regrid_record(q)
        assert rg["lev"] == ro["lev"] and rg["time"] == ro["time"]
        mism += int(np.count_nonzero(rg["mask"] != ro["mask"]))
        cells += rg["mask"].size
    print("FP32 hierarchy: rel L2 per (step, level)", errors,
          f"tag mismatches {mism} of {cells} cells")
    # a truncation error is the difference of two nearly equal values, so
    # its FP32 rounding (about 1e-7 of the field) can move a cell whose
    # error lies within about 1e-5 relative of te_crit across it (none of
    # 77,824 when measured)
    assert mism <= cells // 1000
    g.close()
    o.close()


def test_fp32_hierarchy_checkpoint_restart(ctx, tmp_path):
    cfg = config(precision=F32, record_regrids=0)
    g = sh.Amr(ctx, cfg, level0(2))
    for _ in range(3):
        g.step(1)
    g.checkpoint(str(tmp_path / "ck"))
    r = sh.Amr.restart(ctx, cfg, str(tmp_path / "ck"))
    for _ in range(2):
        g.step(1)
        r.step(1)
    assert g.info() == r.info()
    for lev in range(g.info()["finest"] + 1):
        assert g.level(lev).boxes == r.level(lev).boxes
        # values and compensations are stored as v - c and split again on
        # restart: identical except where a compensation sat on a rounding tie
        assert rel_l2(r.level(lev).read(), g.level(lev).read()) <= 1e-8
    g.close()
    r.close()


def test_fp64_only_operations_refuse_fp32_levels(ctx):
    lv = sh.Level.periodic(ctx, "AxionStringsLap1", 16, 1, precision=F32)
    lv.write(_state(16, 8.0, 1))
    with pytest.raises(sh.ShError) as e:
        lv.rhs(1.0, 0, 0.0625, 0.25, params=[1.0, 0.0])
    assert e.value.code == _lib.SH_ERR_UNSUPPORTED
    with pytest.raises(sh.ShError):
        lv.advance(sh.LEAPFROG, 0.0625, 0.25, params=[1.0, 0.0])
    lv.close()
    with pytest.raises(sh.ShError):
        sh.Level.periodic(ctx, "AxionStringsLap1", 16, 1, with_gw=True, precision=F32)


def _fopt_state(N, L, seed):
    """FirstOrderPhaseTransition + GW state (level order) of FP32 numbers."""
    s = np.zeros((14, N, N, N))
    kmax = 0.5 * np.pi * N / L
    s[0] = 0.5 + 0.3 * ic.gaussian_field(N, L, kmax, seed)
    s[1] = 0.1 * ic.gaussian_field(N, L, kmax, seed + 1)
    for q in range(12):
        s[2 + q] = 1e-3 * ic.gaussian_field(N, L, kmax, seed + 2 + q)
    return s.astype(np.float32).astype(np.float64)


def test_fp32_fopt_level_against_ensemble_and_oracle(ctx, oracle):
    """FirstOrderPhaseTransition + GW on FP32 levels (leapfrog): one box and
    eight boxes give the same bits, within 1e-6 of the FP32 ensemble kernel
    of the same equations (the same FP32 arithmetic in a shared-memory ring)
    and within 5e-6 of the FP64 oracle after 10 steps."""
    N, dx, dt, steps = 32, 0.25, 0.05, 10
    q = [-0.2, 0.5, -0.6]
    st = _fopt_state(N, N * dx, 21)
    E = sh.Ensemble(ctx, sh.FAMILY_FOPT_GW, F32, [N], [dx], q + [0.0])
    E.write(0, st)
    E.set_time(0.0)
    E.step(dt, steps)
    ens = np.asarray(E.read(0)).ravel()
    E.close()
    outs = []
    for max_grid in (0, 16):
        lv = sh.Level.periodic(ctx, "FirstOrderPhaseTransition", N, 2, max_grid=max_grid,
                               with_gw=True, precision=F32)
        lv.write(st)
        lv.set_time(0.0)
        for _ in range(steps):
            lv.advance(sh.LEAPFROG, dt, dx, params=[0.0, *q, 0.0, 0.0, 0.0])
        outs.append(lv.read().ravel())
        lv.close()
    assert np.array_equal(outs[0], outs[1])
    assert rel_l2(outs[0], ens) <= 1e-6, rel_l2(outs[0], ens)
    ref = oracle.evolve_periodic("FirstOrderPhaseTransition", sh.LEAPFROG, st, t0=0.0, dt=dt,
                                 dx=dx, nsteps=steps, params=[0.0, *q, 0.0, 0.0, 0.0],
                                 with_gw=True, nghost=2).ravel()
    e = rel_l2(outs[0], ref)
    eu = rel_l2(outs[0].reshape(14, -1)[2:], ref.reshape(14, -1)[2:])
    print(f"FP32 FOPT level against FP64: fields {e:.2e}, GW tensor {eu:.2e}")
    assert e <= 5e-6 and eu <= 5e-5


def test_fp32_fopt_bubbles_and_hierarchy_against_fp64_oracle(ctx):
    """Bubbles injected into an FP32 FirstOrderPhaseTransition + GW level
    agree with the FP64 level's to FP32 rounding; an FP32 hierarchy of that
    project (leapfrog, truncation-error tags scaled by level-0 maxima) keeps
    the FP64 oracle's levels and boxes, fields within 1e-5 per level."""
    from tests.oracle_lib import oracle_add_bubbles
    N0, L = 16, 8.0
    nb = 60
    r = np.arange(nb) / 8.0
    prof = np.stack([0.5 * (1 - np.tanh((r - 2.0) / 0.7)), np.zeros(nb)])
    st = np.zeros((14, N0, N0, N0))
    st[2:8] = 1e-3 * np.stack([ic.gaussian_field(N0, L, 3.0, 50 + q) for q in range(6)])
    st = st.astype(np.float32).astype(np.float64)
    centres = np.array([[4.1, 3.9, 4.2]])
    a = sh.Level.periodic(ctx, "FirstOrderPhaseTransition", N0, 2, with_gw=True, precision=F32)
    a.write(st)
    a.add_bubbles(centres, prof, 8.0, 7.0, L / N0)
    want = oracle_add_bubbles(st, centres.tolist(), prof, 8.0, 7.0, L / N0)
    assert rel_l2(a.read(), want) <= 1e-7
    a.close()
    lb = 0.8
    num = 3.0 + np.sqrt(9.0 - 8.0 * lb)
    params = [0.0, -1.0, 3.0 * num / (4.0 * lb), -num * num / (8.0 * lb), 0.0, 0.0, 0.0]
    te = [1e-2, 1e-2] + [1e300] * 12
    kw = dict(N0=N0, L=L, cfl=0.2, t_start=0.0, nghost=2, max_level=2, blocking_factor=8,
              max_grid_size=16, n_error_buf=1, regrid_dt=0.0, te_crit=te, params=params,
              with_gw=1, integrator=sh.LEAPFROG, params_mod_norm0=1, record_regrids=0,
              max_local_regrids=0)
    g = sh.Amr(ctx, sh.amr_config("FirstOrderPhaseTransition", precision=F32, **kw), want)
    o = OracleAmr(sh.amr_config("FirstOrderPhaseTransition", **kw), want)
    for step in range(5):
        g.step(1)
        o.step(1)
        assert g.info()["finest"] == o.info()["finest"], step
        for lev in range(g.info()["finest"] + 1):
            assert g.level(lev).boxes == o.boxes(lev), (step, lev)
            e = rel_l2(g.level(lev).read(), o.read(lev)[0])
            assert e <= 1e-5, (step, lev, e)
    assert g.info()["finest"] >= 1
    g.close()
    o.close()


def test_fp32_hierarchy_local_regrids_against_fp64_oracle(ctx):
    """Local regrids on an FP32 hierarchy (blocks added next to coarse/fine
    boundaries, both time levels of the new boxes interpolated) take the FP64
    oracle's decisions: the same boxes after every coarse step, fields
    within 2e-6."""
    kw = dict(record_regrids=0, regrid_dt=0.125, max_local_regrids=10)
    g = sh.Amr(ctx, config(precision=F32, **kw), level0(1))
    o = OracleAmr(config(**kw), level0(1))
    g.set_trace(True)
    o.set_trace(True)
    for step in range(10):
        g.step(1)
        o.step(1)
        assert g.info()["finest"] == o.info()["finest"], step
        for lev in range(g.info()["finest"] + 1):
            assert g.level(lev).boxes == o.boxes(lev), (step, lev)
            e = rel_l2(g.level(lev).read(), o.read(lev)[0])
            assert e <= 2e-6, (step, lev, e)
    assert g.trace() == o.trace()
    assert len(g.level(2).boxes) == 66  # level 2 grew by a block, as in the FP64 test
    g.close()
    o.close()
