"""Checkpoint and restart of an AMR hierarchy (csrc/sh_checkpoint.h, the
shamr::Driver's checkpoint/restart), through the oracle's hierarchy on the
CPU:

* Meta.hdf5 holds the reference's header datasets (Checkpoint::Write,
  source/output_types/checkpoint.cpp:18-98) with the values of the
  hierarchy, readable by the tests' parser of the HDF5 specification;
* a hierarchy restarted from the folder and stepped on equals, bit for bit
  (fields, boxes, times, regrid decisions), the hierarchy that was
  checkpointed and stepped on without stopping;
* a folder whose grid does not match the configuration is refused.
"""
import numpy as np
import pytest

from tests import hdf5_read
from tests.amr_common import config, level0
from tests.oracle_lib import OracleAmr


def _same(a, b):
    assert a.info() == b.info()
    for lev in range(a.info()["finest"] + 1):
        assert a.boxes(lev) == b.boxes(lev)
        for which in (0, 1):
            da, ta = a.read(lev, which)
            db, tb = b.read(lev, which)
            assert ta == tb
            assert np.array_equal(da, db)


@pytest.mark.parametrize("cfg_kw", [dict(), dict(te_crit=[1e300] * 4)])
def test_restart_continues_bit_for_bit(tmp_path, cfg_kw):
    kw = dict(record_regrids=0, **cfg_kw)
    a = OracleAmr(config(**kw), level0(3))
    a.step(3)
    assert a.info()["finest"] >= 1
    a.checkpoint(tmp_path)
    meta = hdf5_read.File(str(tmp_path / "Meta.hdf5"))
    h = meta["Header"]
    info = a.info()
    assert h[2] == info["finest"] and h[3] == 16 and h[4] == 2 and h[5] == 4
    assert h[0] == a.read(0)[1]
    assert list(meta["blocking_factors"]) == [8.0] * (info["finest"] + 1)
    assert len(meta["isteps"]) == info["finest"] + 1 and meta["isteps"][0] == 3
    assert list(meta["next_id"]) == [1.0] and meta["last_time_written"][0] == h[0]
    b = OracleAmr.restart(config(**kw), tmp_path)
    _same(a, b)
    a.step(3)
    b.step(3)
    _same(a, b)
    a.close()
    b.close()


def test_restart_refuses_another_grid(tmp_path):
    a = OracleAmr(config(record_regrids=0), level0(1))
    a.step(2)
    a.checkpoint(tmp_path)
    a.close()
    with pytest.raises(RuntimeError):
        OracleAmr.restart(config(record_regrids=0, max_level=1), tmp_path)
