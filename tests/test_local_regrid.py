"""Local regrids (LocalRegrid, source/local_regrid/local_regrid.cpp) in the
AMR time stepper, through the oracle's hierarchy on the CPU:

* with the reference's defaults (10 attempts, volume thresholds 1.05 and
  1.1) regrids after the first one are attempted locally: the hierarchy
  keeps every existing box and appends blocking-factor-aligned boxes, each
  inside the domain, and the levels stay nested (every fine box inside the
  coarse level's boxes, refined);
* a weak volume threshold of 1 disables them (LocalRegrid::Prechecks), and
  every regrid is global;
* a checkpoint taken between local regrids restarts bit for bit.
"""
import numpy as np
import pytest

from tests.amr_common import config, level0
from tests.oracle_lib import OracleAmr


def _covered(boxes, ratio, i, j, k):
    return any(all(lo[d] * ratio <= (i, j, k)[d] <= hi[d] * ratio + ratio - 1 for d in range(3))
               for lo, hi in boxes)


def test_local_regrids_keep_boxes_and_nesting():
    o = OracleAmr(config(record_regrids=0, regrid_dt=0.125, max_local_regrids=10), level0(1))
    o.set_trace(True)
    before = None
    grew = 0
    for step in range(10):
        o.step(1)
        fin = o.info()["finest"]
        now = [o.boxes(l) for l in range(fin + 1)]
        events = [e for e in o.trace() if e[0] in ("regrid", "local_regrid")]
        if before is not None and events and events[-1][0] == "local_regrid":
            for l in range(1, min(len(before), len(now))):
                assert now[l][: len(before[l])] == before[l]
                grew += len(now[l]) > len(before[l])
        for l in range(1, fin + 1):
            N = 16 << l
            cover = np.zeros((N, N, N), dtype=np.int32)
            for lo, hi in now[l]:
                cover[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] += 1
            assert cover.max() == 1  # disjoint boxes
            for lo, hi in now[l]:
                assert all(x % 8 == 0 for x in lo) and all((x + 1) % 8 == 0 for x in hi)
                # corners of every fine box lie in the coarse level
                for c in ((lo[0], lo[1], lo[2]), (hi[0], hi[1], hi[2])):
                    assert _covered(now[l - 1], 1, c[0] // 2, c[1] // 2, c[2] // 2)
        before = now
    kinds = {e[0] for e in o.trace()}
    assert "local_regrid" in kinds and "regrid" in kinds
    assert grew >= 1
    o.close()


def test_weak_threshold_of_one_disables_local_regrids():
    o = OracleAmr(config(record_regrids=0, volume_threshold_weak=1.0, max_local_regrids=10), level0(5))
    o.set_trace(True)
    o.step(6)
    kinds = {e[0] for e in o.trace()}
    assert "local_regrid" not in kinds and "regrid" in kinds
    o.close()


def test_checkpoint_between_local_regrids_restarts_exactly(tmp_path):
    kw = dict(record_regrids=0, regrid_dt=0.125, max_local_regrids=10)
    a = OracleAmr(config(**kw), level0(1))
    a.step(4)
    a.checkpoint(tmp_path)
    b = OracleAmr.restart(config(**kw), tmp_path)
    a.step(5)
    b.step(5)
    assert a.info() == b.info()
    for lev in range(a.info()["finest"] + 1):
        assert a.boxes(lev) == b.boxes(lev)
        assert np.array_equal(a.read(lev)[0], b.read(lev)[0])
    a.close()
    b.close()
