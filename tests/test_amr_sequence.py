"""Order of operations of the AMR time stepper (csrc/sh_amr_driver.h), run
through the oracle's hierarchy, against sledgehamr's TimeStepper:

* a known-answer sequence written out by hand from source/time_stepper.cpp
  (Advance :90-133, SynchronizeLevels :140-162, ScheduleRegrid :221-295,
  DoRegridIfScheduled :301-311, DoRegrid :346-397) and
  source/regrid_scheduler.cpp for the first four coarse steps of a
  hierarchy with a shadow level that refines everywhere (every cell's
  truncation error passes te_crit = 0), regrid_dt = 0, max_level 2;
* the same with local regrids (LocalRegrid::AttemptRegrid before every
  global regrid, source/local_regrid/local_regrid.cpp:22-401);
* an independent restatement of the same functions (tests/timestepper_model.py)
  over longer runs, with and without the shadow hierarchy, with the regrid
  interval, with the project's CreateLevelIf gate and with local regrids.
Times are compared exactly: both sides add the same doubles in the same
order."""
import pytest

from tests.amr_common import config, level0
from tests.oracle_lib import OracleAmr
from tests.timestepper_model import DBL_MAX, TimeStepperModel

T, D = 3.0, 0.0625      # t_start, coarse dt (dx0 = 0.25, cfl 0.25)
H, Q = D / 2, D / 4     # level 1 and level 2 steps

# TimeStepper on a hierarchy refined everywhere, by hand:
KAT = [
    # coarse step 1: no regrid yet (grid_old[0] undefined, :281-283)
    ("advance", 0, T),
    # step 2: regrid scheduled for the end of this step with a shadow level
    ("schedule", 0, T + 2 * D), ("shadow", -1, T + 2 * D), ("advance", 0, T + D),
    ("truncation_errors", 0, T + 2 * D), ("regrid", 0, T + 2 * D),      # level 1 made
    # step 3: level 1 sub-steps; its odd step schedules (lowest level stays 0)
    ("schedule", 0, T + 3 * D), ("shadow", -1, T + 3 * D), ("advance", 0, T + 2 * D),
    ("advance", 1, T + 2 * D),
    ("schedule", 1, T + 3 * D), ("advance", 1, T + 2 * D + H),
    ("truncation_errors", 1, T + 3 * D), ("truncation_errors", 0, T + 3 * D),
    ("regrid", 0, T + 3 * D),                                              # level 2 made
    # step 4: two level-2 sub-steps per level-1 step; averaging down after
    # the first level-1 step, truncation errors on every level at the end
    ("schedule", 0, T + 4 * D), ("shadow", -1, T + 4 * D), ("advance", 0, T + 3 * D),
    ("advance", 1, T + 3 * D),
    ("advance", 2, T + 3 * D), ("advance", 2, T + 3 * D + Q),
    ("average_down", 1, T + 3 * D + H),
    ("schedule", 1, T + 4 * D), ("advance", 1, T + 3 * D + H),
    ("advance", 2, T + 3 * D + H), ("advance", 2, T + 3 * D + H + Q),
    ("truncation_errors", 2, T + 4 * D), ("truncation_errors", 1, T + 4 * D),
    ("truncation_errors", 0, T + 4 * D), ("regrid", 0, T + 4 * D),
]


def _run(cfg_kw, steps, seed=0):
    o = OracleAmr(config(**cfg_kw), level0(seed))
    o.set_trace(True)
    finest = []
    for _ in range(steps):
        o.step(1)
        finest.append(o.info()["finest"])
    tr = o.trace()
    o.close()
    return tr, finest


# The same hierarchy with local regrids (LocalRegrid::AttemptRegrid before
# every global regrid, local_regrid.cpp:22-401): the regrid of step 2 creates
# level 1 globally (a level above is needed to grow locally); from step 3 on
# level 1 covers the domain, so the local regrid finds no coarse/fine
# boundary to push, succeeds without adding boxes, and level 2 is not made.
KAT_LOCAL = KAT[:14] + [
    # step 3 as above up to the regrid, which is local
    ("local_regrid", 0, T + 3 * D),
    # step 4: level 1 is still the finest level
    ("schedule", 0, T + 4 * D), ("shadow", -1, T + 4 * D), ("advance", 0, T + 3 * D),
    ("advance", 1, T + 3 * D),
    ("schedule", 1, T + 4 * D), ("advance", 1, T + 3 * D + H),
    ("truncation_errors", 1, T + 4 * D), ("truncation_errors", 0, T + 4 * D),
    ("local_regrid", 0, T + 4 * D),
]
assert KAT_LOCAL[13] == ("truncation_errors", 0, T + 3 * D)


def test_time_stepper_known_answer_sequence():
    tr, finest = _run(dict(te_crit=[0.0] * 4, regrid_dt=0.0, string_width_threshold=0.0,
                           max_local_regrids=0), 4)
    assert finest == [0, 1, 2, 2]
    assert tr == KAT


def test_time_stepper_known_answer_sequence_with_local_regrids():
    tr, finest = _run(dict(te_crit=[0.0] * 4, regrid_dt=0.0, string_width_threshold=0.0,
                           max_local_regrids=10), 4)
    assert finest == [0, 1, 1, 1]
    assert tr == KAT_LOCAL


def _model(cfg_kw, grows=lambda lev, t: True):
    c = dict(N0=16, L=4.0, cfl=0.25, t_start=3.0, max_level=2, regrid_dt=0.0,
             string_width_threshold=2.0, max_local_regrids=0)
    c.update({k: v for k, v in cfg_kw.items() if k in c})
    shadow = any(x != DBL_MAX for x in cfg_kw.get("te_crit", [DBL_MAX]))
    return TimeStepperModel(c["N0"], c["L"], c["cfl"], c["t_start"], c["max_level"],
                            c["regrid_dt"], shadow, c["string_width_threshold"], grows=grows,
                            max_local_regrids=c["max_local_regrids"])


@pytest.mark.parametrize("cfg_kw", [
    # shadow hierarchy, regrid every coarse step where possible
    dict(te_crit=[0.0] * 4, regrid_dt=0.0, string_width_threshold=0.0),
    # shadow hierarchy with a regrid interval of three coarse steps
    dict(te_crit=[0.0] * 4, regrid_dt=3 * 0.0625, string_width_threshold=0.0),
    # the project's gate: level 2 needs eta >= 5.66, so it never appears here
    dict(te_crit=[0.0] * 4, regrid_dt=0.0, string_width_threshold=1.0),
    # one refinement level only
    dict(te_crit=[0.0] * 4, regrid_dt=0.0, string_width_threshold=0.0, max_level=1),
    # no shadow hierarchy: regrids at the start of steps (NoShadowRegrid)
    dict(te_crit=[DBL_MAX] * 4, regrid_dt=0.0, string_width_threshold=0.0),
    dict(te_crit=[DBL_MAX] * 4, regrid_dt=2 * 0.0625, string_width_threshold=0.0),
    # local regrids with a small attempt budget: global regrids after every
    # third attempt (the hierarchy refined everywhere never needs new boxes)
    dict(te_crit=[0.0] * 4, regrid_dt=0.0, string_width_threshold=0.0, max_local_regrids=2),
])
def test_time_stepper_sequence_equals_restated_model(cfg_kw):
    cfg_kw = dict(cfg_kw)
    cfg_kw.setdefault("max_local_regrids", 0)
    steps = 7
    tr, finest = _run(cfg_kw, steps, seed=4)
    m = _model(cfg_kw)
    mf = []
    for _ in range(steps):
        m.step()
        mf.append(m.finest)
    assert finest == mf
    assert tr == m.events
    assert max(finest) >= 1
