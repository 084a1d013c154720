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


@pytest.mark.parametrize("integrator", [sh.RKN4, sh.LSSSPRK3])
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
    assert g.info()["finest"] == 2
    for q in range(g.info()["nregrids"]):
        rg, ro = g.regrid_record(q), o.regrid_record(q)
        assert rg["lev"] == ro["lev"] and rg["time"] == ro["time"]
        assert rg["tagged_boxes"] == ro["tagged_boxes"]
        assert np.array_equal(rg["mask"], ro["mask"])
        assert rg["new_boxes"] == ro["new_boxes"]
    g.close()
    o.close()
