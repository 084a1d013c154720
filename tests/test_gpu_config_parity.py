"""Parity at the sizes of the benchmark configurations (CUDA path through the
C ABI against the oracle, same seeded inputs):

* the 128^3 single level (L = 32, seed 0, |k| <= 1, RKN4, dt = 0.0625,
  eta0 = 0.1), 10 steps, for the configured project variant
  (AxionStringsLap1: 7-point Laplacian, lambda = 1, no constant) and for the
  verbatim AxionStrings kernel: fields within 1e-12 relative L2;
* the 256^3 AMR hierarchy (L = 64, 4th-order Laplacian, winding plus
  truncation-error tags with te_crit 1e-3, shadow level) stepped in lockstep
  up to and including the regrid that creates level 1: identical regrid
  decisions, tag masks bit-exact, the same new boxes, fields within 1e-12;
* FirstOrderPhaseTransition with the GW tensor on 384^3 (L = 96, leapfrog,
  dt = 0.05, lambda-bar 0.8, the benchmark's 64 tanh bubbles injected at
  t = 0), 10 steps: fields within 1e-12 (the tensor block separately), and
  the GW spectrum (projection type 2, binned and unbinned) within 1e-10 per
  bin of the numpy restatement of the oracle's spectrum
  (tests/gw_numpy.py) on the oracle's fields.
"""
import numpy as np
import pytest

import bench
import sledgehamr_gb300 as sh
from sledgehamr_gb300 import ic
from tests import gw_numpy
from tests.conftest import rel_l2
from tests.oracle_lib import OracleAmr, oracle_add_bubbles

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-12


@pytest.mark.parametrize("project,params,nghost", [
    ("AxionStringsLap1", [1.0, 0.0], 1),  # the configured variant
    ("AxionStrings", [], 2),              # the reference's kernel as written
])
def test_single_level_128_ten_steps_vs_oracle(ctx, oracle, project, params, nghost):
    st = ic.axion_string_ic(128, 32.0, kmax=1.0, seed=0)
    kw = dict(t0=0.1, dt=0.0625, dx=0.25, nsteps=10, params=params, nghost=nghost)
    gpu = ctx.evolve_periodic(project, sh.RKN4, st, **kw)
    ref = oracle.evolve_periodic(project, sh.RKN4, st, **kw)
    assert rel_l2(gpu, ref) <= FIELD_TOL
    assert rel_l2(gpu[2:], ref[2:]) <= FIELD_TOL  # momenta


def test_amr_256_first_regrid_vs_oracle(ctx):
    cfg = dict(bench.AMR)
    kw = dict(N0=cfg["N0"], L=cfg["L"], cfl=cfg["cfl"], t_start=cfg["t_start"],
              nghost=cfg["nghost"], max_level=cfg["max_level"],
              blocking_factor=cfg["blocking_factor"], max_grid_size=cfg["max_grid_size"],
              n_error_buf=cfg["n_error_buf"], regrid_dt=cfg["regrid_dt"],
              te_crit=[cfg["te_crit"]] * 4, params=cfg["params"],
              string_width_threshold=cfg["string_width_threshold"], record_regrids=1)
    state = ic.axion_string_ic(cfg["N0"], cfg["L"], kmax=1.0, seed=0)
    g = sh.Amr(ctx, sh.amr_config(cfg["project"], **kw), state)
    o = OracleAmr(sh.amr_config(cfg["project"], **kw), state)
    steps = 0
    while g.info()["finest"] < 1 and steps < 60:
        g.step(1)
        o.step(1)
        steps += 1
        assert g.info() == o.info(), steps
    assert g.info()["finest"] == 1
    # every regrid so far (those before level 1 found no cells to refine)
    for q in range(g.info()["nregrids"]):
        rg, ro = g.regrid_record(q), o.regrid_record(q)
        assert (rg["lev"], rg["time"]) == (ro["lev"], ro["time"])
        assert np.array_equal(rg["mask"], ro["mask"])
        assert rg["new_boxes"] == ro["new_boxes"]
    last = g.regrid_record(g.info()["nregrids"] - 1)
    assert last["mask"].sum() > 0 and len(last["new_boxes"]) > 0
    for lev in range(2):
        gd = g.level(lev).read()
        od, _ = o.read(lev)
        assert g.level(lev).boxes == o.boxes(lev)
        assert rel_l2(gd, od) <= FIELD_TOL
    g.close()
    o.close()


def test_fopt_gw_384_ten_leapfrog_steps_and_spectrum(ctx, oracle):
    f = bench.FOPT
    N, dx, dt = f["N"], f["dx"], f["dt"]
    xyz, _, prof, Lcut = bench.fopt_bubbles()
    q = bench.lambda_bar_params(f["lambda_bar"])
    params = [0.0, *q, 0.0, 0.0, 0.0]
    state = oracle_add_bubbles(np.zeros((14, N, N, N)), xyz, prof, f["inv_dx"], Lcut, dx)
    lv = sh.Level.periodic(ctx, "FirstOrderPhaseTransition", N, 2, max_grid=f["max_grid"],
                           with_gw=True)
    lv.write(np.zeros((14, N, N, N)))
    lv.add_bubbles(xyz, prof, f["inv_dx"], Lcut, dx)
    assert np.array_equal(lv.read(), state)  # injection is bit-exact
    lv.set_time(0.0)
    for _ in range(10):
        lv.advance(sh.LEAPFROG, dt, dx, params=params)
    gpu = lv.read()
    ref = oracle.evolve_periodic("FirstOrderPhaseTransition", sh.LEAPFROG, state, t0=0.0,
                                 dt=dt, dx=dx, nsteps=10, params=params, with_gw=True,
                                 nghost=2, max_grid=f["max_grid"])
    assert rel_l2(gpu, ref) <= FIELD_TOL
    assert rel_l2(gpu[2:], ref[2:]) <= FIELD_TOL
    comps = [ref[2 + 6 + d] for d in (0, 3, 4, 1, 5, 2)]  # du_xx du_xy du_xz du_yy du_yz du_zz
    del ref, state, gpu
    for unbinned in (False, True):
        bins, ks = lv.gw_spectrum(zero_padding=1, projection_type=2, unbinned=unbinned)
        rb, rks = gw_numpy.gw_spectrum(comps, 1, 2, unbinned, oracle.index_to_k,
                                       oracle.unique_k2)
        assert np.array_equal(ks, rks)
        scale = np.abs(rb).max()
        assert scale > 0
        assert np.all(np.abs(bins - rb) <= 1e-10 * np.abs(rb) + 1e-14 * scale)
    lv.close()
