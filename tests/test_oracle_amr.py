"""The AMR hierarchy on the oracle: levels appear, stay properly nested and
aligned, and coarse cells under finer levels hold their averages."""
import numpy as np

from tests.amr_common import boxes_layout_to_levelwise, config, level0
from tests.oracle_lib import OracleAmr


def covered(boxes, i, j, k):
    return any(lo[0] <= i <= hi[0] and lo[1] <= j <= hi[1] and lo[2] <= k <= hi[2]
               for lo, hi in boxes)


def test_oracle_amr_levels_nesting_and_average_down():
    cfg = config()
    o = OracleAmr(cfg, level0())
    seen_finest = 0
    for _ in range(3):
        o.step(1)
        seen_finest = max(seen_finest, o.info()["finest"])
    info = o.info()
    assert seen_finest == 2 and info["nregrids"] >= 3
    for lev in range(1, info["finest"] + 1):
        N = 16 << lev
        for lo, hi in o.boxes(lev):
            for d in range(3):
                assert lo[d] % 8 == 0 and (hi[d] + 1) % 8 == 0 and 0 <= lo[d] <= hi[d] < N
                assert hi[d] - lo[d] + 1 <= 16
        # proper nesting: every cell's parent lies on the level below
        crse = o.boxes(lev - 1)
        for lo, hi in o.boxes(lev):
            for k in (lo[2], hi[2]):
                for j in (lo[1], hi[1]):
                    for i in (lo[0], hi[0]):
                        assert covered(crse, i // 2, j // 2, k // 2)
    # coarse cells under level 1 equal the 2x2x2 average of level 1
    fine, _ = o.read(1)
    crse, _ = o.read(0)
    fb = boxes_layout_to_levelwise(fine, o.boxes(1), 4)
    cb = boxes_layout_to_levelwise(crse, o.boxes(0), 4)
    (clo, chi), = o.boxes(0)
    for (lo, hi), f in zip(o.boxes(1), fb):
        avg = f.reshape(4, f.shape[1] // 2, 2, f.shape[2] // 2, 2, f.shape[3] // 2, 2).mean(
            axis=(2, 4, 6))
        c = cb[0][:, lo[2] // 2:(hi[2] + 1) // 2, lo[1] // 2:(hi[1] + 1) // 2,
                  lo[0] // 2:(hi[0] + 1) // 2]
        assert np.allclose(c, avg, rtol=0, atol=1e-13)
    assert np.isfinite(fine).all() and np.isfinite(crse).all()
    o.close()
