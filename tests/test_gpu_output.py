"""Level and slice files written from levels on the GPU (sh_output_level,
sh_output_slices) equal the oracle's restatement of sledgehamr's
LevelWriter and Slices on the same cells, for a standalone level (data from
time level NEW, truncation errors from OLD) and for every level of an AMR
hierarchy (full_box layout, Level_<lev>/0.hdf5)."""
import os

import numpy as np
import pytest

import sledgehamr_gb300 as sh
from oracle import output_oracle as oo
from sledgehamr_gb300 import output
from tests import hdf5_read
from tests.amr_common import config, level0
from tests.test_output_files import _compare, _level

pytestmark = pytest.mark.gpu


def test_level_and_slice_files_match_oracle(ctx, tmp_path):
    rng = np.random.default_rng(11)
    boxes = _level(rng, N=32, nbox=6)
    L = sh.Level(ctx, "AxionStrings", boxes, (0, 0, 0), (31, 31, 31), 2)
    new = rng.standard_normal(L.nvalid * L.ncomp)
    old = np.abs(rng.standard_normal(L.nvalid * L.ncomp))
    L.write(new, sh.SH_NEW, layout=1)
    L.write(old, sh.SH_OLD, layout=1)
    L.set_time(2.0, sh.SH_NEW)
    L.set_time(1.75, sh.SH_OLD)
    names = output.comp_names("AxionStrings")
    for precision, ds in [(32, 1), (64, 2), (32, 4)]:
        p = str(tmp_path / f"l{precision}_{ds}.hdf5")
        output.level_file(ctx, L, 1, True, ds, precision).write(p)
        want = oo.level_datasets(boxes, new, names, 2.0, 1, 32, "data", False, ds, precision)
        want.update(oo.level_datasets(boxes, old, names, 1.75, 1, 32, "te", True, ds,
                                      precision))
        _compare(hdf5_read.File(p), want)
    loc = (0.3, 0.5, 0.71)
    p = str(tmp_path / "s.hdf5")
    output.slices_file(ctx, L, 1, True, loc).write(p)
    want = oo.slices_datasets(boxes, new, names, 2.0, 1, 32, False, loc)
    want.update(oo.slices_datasets(boxes, old, names, 1.75, 1, 32, True, loc))
    _compare(hdf5_read.File(p), want)
    L.close()


def test_amr_full_box_files(ctx, tmp_path):
    g = sh.Amr(ctx, config(), level0())
    g.step(3)
    finest = g.info()["finest"]
    assert finest >= 1
    levels = [g.level(lev) for lev in range(finest + 1)]
    folder = output.output_folder(str(tmp_path), "full_box", 0)
    paths = output.write_boxes(folder, ctx, levels, downsample=1, precision=64)
    names = output.comp_names("AxionStringsLap2")
    for lev, (lv, p) in enumerate(zip(levels, paths)):
        assert p == os.path.join(folder, f"Level_{lev}", "0.hdf5")
        N = lv.domain[1][0] - lv.domain[0][0] + 1
        want = oo.level_datasets(lv.boxes, lv.read(sh.SH_NEW), names, lv.time()[0], finest,
                                 N, "data", False, 1, 64)
        _compare(hdf5_read.File(p), want)
    g.close()
