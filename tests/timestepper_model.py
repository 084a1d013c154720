"""A model of sledgehamr's AMR time stepper that records only the order of
its operations (test infrastructure; no field data).

It restates, from the reference's source:
  TimeStepper::Advance ........... source/time_stepper.cpp:90-133
  TimeStepper::SynchronizeLevels . time_stepper.cpp:140-162
  TimeStepper::SynchronizeTimes .. time_stepper.cpp:168-171
  TimeStepper::ScheduleRegrid .... time_stepper.cpp:221-295
  TimeStepper::DoRegridIfScheduled time_stepper.cpp:301-311
  TimeStepper::NoShadowRegrid .... time_stepper.cpp:317-339
  TimeStepper::DoRegrid .......... time_stepper.cpp:346-397 (local regrid
                                   attempt, then the global regrid)
  LocalRegrid prechecks .......... source/local_regrid/local_regrid.cpp:109-146
  RegridScheduler ................ source/regrid_scheduler.cpp
  Integrator::Advance ............ source/integrators/integrator.cpp:11-31
                                   (swap, t_new = t_old + dt, istep + 1)
  LevelData defaults ............. source/level_data.h:22-66 (t = -DBL_MAX,
                                   istep = 0)
  MakeNewLevelFromCoarse / RemakeLevel / CreateShadowLevel
                                   source/sledgehamr.cpp:149-251
  AxionStrings CreateLevelIf ..... projects/AxionStrings/cosmology.h:25-27,46-48
and AMReX's AmrCore::regrid as sledgehamr uses it (levels lbase+1 and up
remade from the tags of the level below, at most one new level per
regrid).  Whether a regrid's tags yield boxes is a parameter (`grows`):
the model does not tag.

Events are (op, level, time) with the same vocabulary as the library's
trace: advance (level, time before the step), schedule (level, the regrid
time), shadow (-1, the shadow level's time after its step), average_down
(coarse level, its time), truncation_errors (level, its time), regrid (base
level, time).
"""
from __future__ import annotations

import math

DBL_MAX = 1.7976931348623157e308


class TimeStepperModel:
    def __init__(self, N0, L, cfl, t_start, max_level, regrid_dt, shadow_hierarchy,
                 string_width_threshold=0.0, string_lambda=1.0, grows=lambda lev, t: True,
                 max_local_regrids=0, local_succeeds=lambda lev, t: True):
        self.max_level = max_level
        self.t_start = t_start
        self.shadow_hierarchy = shadow_hierarchy
        self.threshold = string_width_threshold
        self.string_lambda = string_lambda
        self.grows = grows
        self.dx = [L / (N0 << l) for l in range(max_level + 1)]
        self.dt = [self.dx[l] * cfl for l in range(max_level + 1)]
        self.regrid_dt = [regrid_dt / 2.0 ** l for l in range(max_level + 1)]
        self.last_regrid_time = [t_start] * (max_level + 1)
        # grid_new / grid_old time and istep per level (level_data.h defaults)
        self.t_new = [t_start] + [-DBL_MAX] * max_level
        self.t_old = [-DBL_MAX] * (max_level + 1)
        self.s_new = [0] * (max_level + 1)
        self.s_old = [0] * (max_level + 1)
        self.finest = 0
        self.schedule: list[list] = []  # [lowest_level, time]
        self.events: list[tuple[str, int, float]] = []
        # LocalRegrid (source/local_regrid/local_regrid.cpp:22-401): attempts
        # since the last global regrid; whether an attempt that passes the
        # prechecks succeeds is a parameter (the model does not tag)
        self.max_local_regrids = max_local_regrids
        self.local_succeeds = local_succeeds
        self.local_attempts = 0

    # ---- RegridScheduler (regrid_scheduler.cpp) -------------------------
    def _find(self, t):
        # std::find with ScheduleEntry::operator== (regrid_scheduler.h:26-29):
        # equal within 1e-12 of the scheduled time
        for q, (_, ts) in enumerate(self.schedule):
            teps = ts * 1e-12
            if ts > t - teps and ts < t + teps:
                return q
        return -1

    def _schedule(self, lev, t):
        q = self._find(t)
        if q < 0:
            self.schedule.append([lev, t])
        else:
            self.schedule[q][0] = min(lev, self.schedule[q][0])

    def _do_regrid(self, lev, t):
        q = self._find(t)
        return q >= 0 and self.schedule[q][0] == lev

    def _need_te(self, lev, t):
        q = self._find(t)
        return q >= 0 and lev >= self.schedule[q][0]

    def _did_regrid(self, t):
        q = self._find(t)
        if q >= 0:
            del self.schedule[q]

    # ---- project hook: AxionStrings CreateLevelIf ------------------------
    def _create_level_if(self, lev, t):
        if lev <= 0 or self.threshold <= 0:
            return True
        width = 1.0 / (math.sqrt(2.0 * self.string_lambda) * t * self.dx[lev - 1])
        return width <= self.threshold

    # ---- TimeStepper -----------------------------------------------------
    def step(self):
        self.advance(0)

    def advance(self, lev):
        if self.shadow_hierarchy:
            self._schedule_regrid(lev)
        else:
            self._no_shadow_regrid(lev)
        self.events.append(("advance", lev, self.t_new[lev]))
        # Integrator::Advance: swap, then new = old + dt, istep + 1
        self.t_old[lev], self.s_old[lev] = self.t_new[lev], self.s_new[lev]
        self.t_new[lev] = self.t_old[lev] + self.dt[lev]
        self.s_new[lev] = self.s_old[lev] + 1
        if lev != self.finest:
            self.advance(lev + 1)
            self.advance(lev + 1)
        self._synchronize_levels(lev)
        self._do_regrid_if_scheduled(lev)
        if lev == 0:  # SynchronizeTimes
            for l in range(1, self.finest + 1):
                self.t_new[l] = self.t_new[0]

    def _synchronize_levels(self, lev):
        te = self._need_te(lev, self.t_new[lev])
        if lev < self.finest and not (self.shadow_hierarchy and te):
            self.events.append(("average_down", lev, self.t_new[lev]))
        if lev >= 1 - int(self.shadow_hierarchy) and te:
            self.events.append(("truncation_errors", lev, self.t_new[lev]))

    def _schedule_regrid(self, lev):
        time, istep = self.t_new[lev], self.s_new[lev]
        if self._do_regrid(lev, time + self.dt[lev]):
            return
        if self.t_old[lev] == time:
            return
        if lev >= self.max_level:
            return
        if istep % 2 == 0 and lev > 0:
            return
        nxt = time + 3.0 * self.dt[lev] if lev > 0 else time + 2.0 * self.dt[lev]
        if not self._create_level_if(lev + 1, nxt):
            return
        if nxt <= self.last_regrid_time[lev] + self.regrid_dt[lev]:
            return
        if lev == 0 and self.t_old[lev] == -DBL_MAX:
            return
        self._schedule(lev, time + self.dt[lev])
        self.events.append(("schedule", lev, time + self.dt[lev]))
        if lev == 0:
            # CreateShadowLevel: level 0's old data advanced by 2 dt0
            self.events.append(("shadow", -1, self.t_old[0] + 2.0 * self.dt[0]))

    def _do_regrid_if_scheduled(self, lev):
        time = self.t_new[lev]
        if not self._do_regrid(lev, time):
            return
        self._regrid(lev, time)
        self._did_regrid(time)

    def _no_shadow_regrid(self, lev):
        time = self.t_new[lev]
        if lev >= self.max_level:
            return
        if time + self.dt[lev] <= self.last_regrid_time[lev] + self.regrid_dt[lev]:
            return
        if not self._create_level_if(lev + 1, time + self.dt[lev]):
            return
        self._regrid(lev, time)

    def _regrid(self, lbase, time):
        # TimeStepper::DoRegrid: LocalRegrid::AttemptRegrid first
        # (Prechecks, local_regrid.cpp:109-146: attempts left, a level above
        # to grow), the global regrid when it does not succeed
        attempt = self.local_attempts < self.max_local_regrids
        self.local_attempts += 1
        if attempt and lbase != self.finest and self.local_succeeds(lbase, time):
            self.events.append(("local_regrid", lbase, time))
            for l in range(lbase, self.finest + 1):
                self.last_regrid_time[l] = time
            return
        self.events.append(("regrid", lbase, time))
        self.local_attempts = 0  # LocalRegrid::DidGlobalRegrid
        top = min(self.finest, self.max_level - 1)
        new_finest = lbase
        for l in range(lbase, top + 1):
            # ErrorEst skips the start time with a shadow hierarchy and levels
            # the project does not want yet (sledgehamr.cpp:207-229)
            tags = not (time == self.t_start and self.shadow_hierarchy) and \
                self._create_level_if(l + 1, time) and self.grows(l, time)
            if not tags:
                break
            f = l + 1
            if f > self.finest:  # MakeNewLevelFromCoarse
                self.t_new[f], self.s_new[f] = time, 0
                self.t_old[f], self.s_old[f] = -DBL_MAX, 0
            # RemakeLevel keeps both time levels' times and steps
            new_finest = f
            if f > self.finest:
                break
        for l in range(self.finest, new_finest, -1):  # ClearLevel
            self.t_new[l], self.t_old[l] = -DBL_MAX, -DBL_MAX
            self.s_new[l] = self.s_old[l] = 0
        self.finest = new_finest
        for l in range(lbase, self.finest + 1):
            self.last_regrid_time[l] = time
