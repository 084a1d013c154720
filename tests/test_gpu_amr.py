"""AMR hierarchy on the GPU against the oracle's hierarchy (same time
stepper, CPU numerics): identical regrid decisions (tag masks bit-exact,
identical new boxes) and per-level fields within 1e-12 relative L2."""
import numpy as np
import pytest

import sledgehamr_gb300 as sh
from tests.amr_common import config, level0
from tests.conftest import rel_l2
from tests.oracle_lib import Oracle, OracleAmr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("integrator", [sh.RKN4, sh.LSSSPRK3, sh.LEAPFROG, sh.RKN5])
def test_amr_matches_oracle(ctx, integrator):
    cfg = config(integrator=integrator)
    g = sh.Amr(ctx, cfg, level0())
    o = OracleAmr(config(integrator=integrator), level0())
    for step in range(3):
        g.step(1)
        o.step(1)
        gi, oi = g.info(), o.info()
        assert gi == oi, (step, gi, oi)
        for lev in range(gi["finest"] + 1):
            gl = g.level(lev)
            assert gl.boxes == o.boxes(lev)
            gd = gl.read()
            od, ot = o.read(lev)
            assert gl.time()[0] == pytest.approx(ot, rel=0, abs=1e-12)
            assert rel_l2(gd, od) <= 1e-12, (step, lev, rel_l2(gd, od))
    assert g.info()["finest"] >= 1
    for q in range(g.info()["nregrids"]):
        rg, ro = g.regrid_record(q), o.regrid_record(q)
        assert rg["lev"] == ro["lev"] and rg["time"] == ro["time"]
        assert rg["tagged_boxes"] == ro["tagged_boxes"]
        assert np.array_equal(rg["mask"], ro["mask"])
        assert rg["new_boxes"] == ro["new_boxes"]
    g.close()
    o.close()


@pytest.mark.parametrize("clustering", [0, 1, 2])
def test_amr_block_tags_match_oracle(ctx, clustering):
    """Without recorded regrids the GPU tags straight to blocks
    (sh_tag_blocks); the hierarchy still equals the oracle's, which coarsens
    its CPU mask on the host."""
    cfg = dict(record_regrids=0, clustering=clustering)
    g = sh.Amr(ctx, config(**cfg), level0(1))
    o = OracleAmr(config(**cfg), level0(1))
    for step in range(3):
        g.step(1)
        o.step(1)
        assert g.info() == o.info()
        for lev in range(g.info()["finest"] + 1):
            assert g.level(lev).boxes == o.boxes(lev)
            od, _ = o.read(lev)
            assert rel_l2(g.level(lev).read(), od) <= 1e-12
    assert g.info()["finest"] >= 1
    g.close()
    o.close()


def test_tag_blocks_equal_coarsened_mask(ctx):
    """sh_tag_blocks equals the host coarsening of sh_tag's mask."""
    import ctypes as C
    from sledgehamr_gb300 import ic
    N = 32
    st = ic.axion_string_ic(N, 8.0, kmax=3.0, seed=5)
    lv = sh.Level.periodic(ctx, "AxionStringsLap1", N, 1, max_grid=8)
    lv.write(st)
    mask, counts, _ = lv.tag(1.0, 0, 0.0625, 0.25)
    for block, buf in ((4, 1), (4, 2), (8, 0)):
        nb = N // block
        blocks = np.zeros(nb ** 3, dtype=np.uint8)
        nt = C.c_longlong()
        ctx.check(ctx.lib.sh_tag_blocks(ctx.h, lv.h, 0, C.c_double(1.0), 0, C.c_double(0.0625),
                                        C.c_double(0.25), None, None, 0, None, 0, block, buf,
                                        C.c_void_p(blocks.ctypes.data), C.byref(nt)),
                  "sh_tag_blocks")
        assert nt.value == counts[0]
        ref = np.zeros((nb, nb, nb), dtype=np.uint8)
        off = 0
        for lo, hi in lv.boxes:
            n = [hi[d] - lo[d] + 1 for d in range(3)]
            m = mask[off: off + n[0] * n[1] * n[2]].reshape(n[2], n[1], n[0])
            off += n[0] * n[1] * n[2]
            for k, j, i in zip(*np.nonzero(m)):
                c = (lo[0] + i, lo[1] + j, lo[2] + k)
                rng = [range((c[d] - buf) // block, (c[d] + buf) // block + 1) for d in range(3)]
                for bz in rng[2]:
                    for by in rng[1]:
                        for bx in rng[0]:
                            ref[bz % nb, by % nb, bx % nb] = 1
        assert np.array_equal(blocks.reshape(nb, nb, nb), ref)
    lv.close()


@pytest.mark.parametrize("norm0", [0, 1])
def test_fopt_gw_amr_with_tag_params_matches_oracle(ctx, norm0):
    """FirstOrderPhaseTransition + GW tensor on an AMR hierarchy (leapfrog,
    truncation-error tags scaled by the field maxima as the
    TruncationModifier parameters: given once, or taken from level 0 at
    every regrid as the project does) against the oracle's hierarchy."""
    from sledgehamr_gb300 import ic
    from tests.oracle_lib import oracle_add_bubbles
    N0, L = 16, 8.0
    nb = 60
    r = np.arange(nb) / 8.0
    prof = np.stack([0.5 * (1 - np.tanh((r - 2.0) / 0.7)), np.zeros(nb)])
    st = np.zeros((14, N0, N0, N0))
    st[2:8] = 1e-3 * np.stack([ic.gaussian_field(N0, L, 3.0, 50 + q) for q in range(6)])
    st = oracle_add_bubbles(st, [[4.1, 3.9, 4.2]], prof, 8.0, 7.0, L / N0)
    n = np.arange(1.0)
    lb = 0.8
    num = 3.0 + np.sqrt(9.0 - 8.0 * lb)
    params = [0.0, -1.0, 3.0 * num / (4.0 * lb), -num * num / (8.0 * lb), 0.0, 0.0, 0.0]
    te = [1e-2, 1e-2] + [1e300] * 12
    pmod = [float(np.abs(st[c]).max()) or 1.0 for c in range(14)]
    kw = dict(N0=N0, L=L, cfl=0.2, t_start=0.0, nghost=2, max_level=2, blocking_factor=8,
              max_grid_size=16, n_error_buf=1, regrid_dt=0.0, te_crit=te, params=params,
              with_gw=1, integrator=sh.LEAPFROG, params_mod=pmod, record_regrids=1,
              params_mod_norm0=norm0)
    g = sh.Amr(ctx, sh.amr_config("FirstOrderPhaseTransition", **kw), st)
    o = OracleAmr(sh.amr_config("FirstOrderPhaseTransition", **kw), st)
    for step in range(5):
        g.step(1)
        o.step(1)
        assert g.info() == o.info()
        for lev in range(g.info()["finest"] + 1):
            assert g.level(lev).boxes == o.boxes(lev)
            od, _ = o.read(lev)
            assert rel_l2(g.level(lev).read(), od) <= 1e-12
    assert g.info()["finest"] >= 1
    g.close()
    o.close()


def test_amr_operation_order_equals_known_answer(ctx):
    """The GPU hierarchy's time stepper performs sledgehamr's operations in
    the order written out by hand from source/time_stepper.cpp
    (tests/test_amr_sequence.py)."""
    from tests.test_amr_sequence import KAT
    g = sh.Amr(ctx, config(te_crit=[0.0] * 4, regrid_dt=0.0, string_width_threshold=0.0,
                           max_local_regrids=0), level0(0))
    g.set_trace(True)
    g.step(4)
    assert g.info()["finest"] == 2
    assert g.trace() == KAT
    g.close()


def test_checkpoint_restart_on_gpu_and_in_the_oracle(ctx, tmp_path):
    """A GPU hierarchy checkpointed after 3 coarse steps (sh_amr_checkpoint)
    and restarted (sh_amr_restart) continues bit for bit like the hierarchy
    that did not stop; the oracle restarted from the same folder takes the
    same regrid decisions and stays within 1e-12 of it."""
    cfg = dict(record_regrids=0)
    g = sh.Amr(ctx, config(**cfg), level0(3))
    g.step(3)
    assert g.info()["finest"] >= 1
    g.checkpoint(str(tmp_path))
    r = sh.Amr.restart(ctx, config(**cfg), str(tmp_path))
    o = OracleAmr.restart(config(**cfg), tmp_path)
    for _ in range(3):
        g.step(1)
        r.step(1)
        o.step(1)
    assert g.info() == r.info() == o.info()
    for lev in range(g.info()["finest"] + 1):
        assert g.level(lev).boxes == r.level(lev).boxes == o.boxes(lev)
        gd = g.level(lev).read()
        assert np.array_equal(gd, r.level(lev).read())
        assert rel_l2(gd, o.read(lev)[0]) <= 1e-12
    g.close()
    r.close()
    o.close()


def test_amr_local_regrids_match_oracle(ctx):
    """Local regrids (LocalRegrid::AttemptRegrid before each global regrid)
    on the GPU hierarchy take the oracle's decisions: the same boxes after
    every coarse step (including a level grown by a block), fields within
    1e-12."""
    kw = dict(record_regrids=0, regrid_dt=0.125, max_local_regrids=10)
    g = sh.Amr(ctx, config(**kw), level0(1))
    o = OracleAmr(config(**kw), level0(1))
    g.set_trace(True)
    o.set_trace(True)
    for step in range(10):
        g.step(1)
        o.step(1)
        assert g.info() == o.info(), step
        for lev in range(g.info()["finest"] + 1):
            assert g.level(lev).boxes == o.boxes(lev), (step, lev)
            assert rel_l2(g.level(lev).read(), o.read(lev)[0]) <= 1e-12
    assert g.trace() == o.trace()
    assert any(e[0] == "local_regrid" for e in g.trace())
    assert len(g.level(2).boxes) == 66  # level 2 grew by one block locally
    g.close()
    o.close()
