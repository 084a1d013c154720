"""Benchmark of the time-stepping hot path: cell-updates/s on one GPU.

Headline (the JSON line's value, e2e, roofline, cpu_baseline): axion
strings, 128^3 periodic single level, L = 32 (dx = 0.25), 2nd-order
(7-point) Laplacian, lambda = 1, RKN4, eta0 = 0.1, dt = 0.25 dx, FP64, on
the drop-in level path (sh_level_advance); one step = one RKN4 step of the
level.  The whole job is 200 steps.

Legs reported beside it under "legs" (each with its own workload, timed
window and errors):
  amr: 256^3 coarse grid (L = 64, dx = 0.25) plus 2 refinement levels
      (ratio 2, blocking factor 8, max grid size 32), 4th-order Laplacian,
      RKN4 with subcycling, tags = plaquette winding OR truncation error
      (te_crit 1e-3, shadow level).  AxionStrings creates level 1 at
      eta ~ 1.9 and level 2 at eta ~ 3.8, so the leg first steps (untimed)
      until the hierarchy holds every level, then times coarse steps with
      all three levels; one step = one coarse step (Advance(0) with every
      finer sub-step, synchronisation and regrid).
  batched_ensemble, fopt_precision, serving: the three chosen forms (FP32 +
      Kahan batched ensemble, FOPT + GW precision form, serving loop).
One cell-update = one valid cell of one level advanced by one full step of
that level, all components.  Seeded band-limited Gaussian initial state
(|k| <= 1, unit variance, Pi = 0).

value   : device-resident state; each timed step bracketed by CUDA events on
          the library's stream, L2 flushed (512 MB write) between timed steps
          outside the events.
e2e     : the whole job through the public C ABI with host buffers: the
          level created and the initial state uploaded from pinned host
          memory, every step, the final state read back to pinned host
          memory (per-step bytes = totals / steps of the job); the median
          of three such jobs.
roofline: the fused stage kernels (Rhs + RKN4 stage update): algorithmic bytes
          of all their launches over their summed duration (CUDA events the
          library records around each launch on its stream), against the
          measured HBM copy bandwidth; fp64_roofline: the same kernels'
          FP64 instruction issue (ncu counts per cell-update) against the
          FP64 FMA rate measured by `--case fp64-peak`.
cpu_baseline: the CPU oracle (FP64 restatement, OpenMP, all host cores) on a
          bounded sample of the same workload.

--impl reference: the reference's CPU path on the host cores (the oracle
port; the reference itself cannot be built without AMReX), on the headline
workload and config; it loads no library of this package.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s"
# Algorithmic HBM words per cell-update of the fused RKN4 schedule as run,
# for 2 position + 2 momentum components: stage i reads the stage state, y0
# and the K_j with a non-zero tableau coefficient, writes K_i and the next
# stage state; the last stage writes y1.  Stage 0: 4 + 2 + 4 = 10; stage 1
# (a_31 = 0: K_0 not read): 4 + 4 + 2 + 4 = 14; final: 4 + 4 + 2 + 2 + 4 =
# 16; 40 FP64 words.
WORDS_PER_CELL_UPDATE = 40
# Measured DRAM traffic of the stage kernels per cell-update (ncu, dram
# bytes read + written of the three launches of one RKN4 step), scaled to a
# launch of the benchmark by the cells it updates.  AMR: level 1 of the AMR
# run at N0 = 128 (5.55 GB for 12,729,344 cells); 128^3 level: the three
# launches of one step of `--case single`, ghost images written by the stage
# kernel (603.1 MB for 2,097,152 cells).
TRAFFIC_B_PER_CELL_UPDATE = {"amr": 436.0, "single": 287.6}
# whole-job end-to-end runs of the 128^3 level (the median is reported)
E2E_JOBS = 3

SINGLE = dict(N=128, L=32.0, project="AxionStringsLap1", params=[1.0, 0.0], nghost=1,
              eta0=0.1, total_steps=200, seed=0)
AMR = dict(N0=256, L=64.0, project="AxionStringsLap2", params=[1.0, 0.0], nghost=2,
           t_start=0.1, cfl=0.25, max_level=2, blocking_factor=8, max_grid_size=32,
           n_error_buf=2, regrid_dt=0.25, te_crit=1e-3, string_width_threshold=1.5,
           t_end=6.0, max_local_regrids=0)


def load_ic():
    """The seeded initial-condition module (numpy only), loaded from its
    file without importing the package, so that the reference arm touches
    no code of the library."""
    spec = importlib.util.spec_from_file_location(
        "sh_ic_standalone", os.path.join(ROOT, "sledgehamr_gb300", "ic.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


ENSEMBLE = dict(nreal=192, sizes=(32, 48, 64, 96, 128), lam=(0.5, 4.0), dx=0.25, eta0=0.1,
                total_steps=94, seed=2024)


def ensemble_spec():
    """Realisation sizes and couplings of the batched-ensemble workload
    (seeded): N uniform in the size set, lambda log-uniform."""
    e = ENSEMBLE
    rng = np.random.default_rng(e["seed"])
    Ns = [int(x) for x in rng.choice(e["sizes"], e["nreal"])]
    lam = np.exp(rng.uniform(np.log(e["lam"][0]), np.log(e["lam"][1]), e["nreal"]))
    return Ns, lam


def ensemble_states(Ns):
    from sledgehamr_gb300 import ic
    dx = ENSEMBLE["dx"]
    return [ic.axion_string_ic(N, N * dx, kmax=1.0, seed=1000 + r) for r, N in enumerate(Ns)]


def run_ensemble_leg(sh, ctx, stream, flush, steps, warmup):
    """Batched ensemble: FP32+Kahan (graph steps, autotuned tiles) against
    the FP64 plain path (one drop-in level per realisation, sh_level_advance)
    and the FP64 batched ensemble on the same realisations.  Each leg runs
    total_steps RKN4 steps; steps [warmup, warmup + steps) are timed with CUDA
    events (L2 flushed between steps; the working set is larger than L2).
    Errors: per-realisation string count and energy of the FP32 run against
    the FP64 plain run at the end, and the relative L2 of the fields."""
    import torch
    e = ENSEMBLE
    Ns, lam = ensemble_spec()
    dx, dt = e["dx"], 0.25 * e["dx"]
    total = max(e["total_steps"], warmup + steps)
    states = ensemble_states(Ns)
    cells = sum(N ** 3 for N in Ns)
    params = np.array([[l, 0.0, 0.0, 0.0] for l in lam]).ravel()

    def timed(step_fn):
        for _ in range(warmup):
            step_fn()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        for a, b in ev:
            flush.zero_()
            a.record(stream)
            step_fn()
            b.record(stream)
        torch.cuda.synchronize()
        ms = float(sum(a.elapsed_time(b) for a, b in ev))
        for _ in range(total - warmup - steps):
            step_fn()
        torch.cuda.synchronize()
        return ms

    out = {}
    # FP32 + Kahan, batched
    t0 = time.perf_counter()
    E32 = sh.Ensemble(ctx, sh.FAMILY_AXION_LAP1, sh.PREC_FP32_KAHAN, Ns, [dx] * len(Ns), params)
    for r, st in enumerate(states):
        E32.write(r, st)
    E32.set_time(e["eta0"])
    nz = E32.tune(dt)
    staging32 = ["registers", "tensor copies"][E32.staging()]
    E32.set_graph(True)
    l0 = E32.kernel_launches()
    ms32 = timed(lambda: E32.step(dt, 1))
    launches32 = E32.kernel_launches() - l0
    e32 = E32.energy()
    s32 = E32.string_count()
    f32 = [E32.read(r) for r in range(len(Ns))]
    info32 = E32.info()
    E32.close()
    wall32 = time.perf_counter() - t0
    # plain FP32 (no compensation), batched: the error the Kahan update removes
    E32p = sh.Ensemble(ctx, sh.FAMILY_AXION_LAP1, sh.PREC_FP32, Ns, [dx] * len(Ns), params)
    for r, st in enumerate(states):
        E32p.write(r, st)
    E32p.set_time(e["eta0"])
    E32p.tune(dt, tile_nz=nz)
    E32p.set_graph(True)
    ms32p = timed(lambda: E32p.step(dt, 1))
    s32p = E32p.string_count()
    f32p = [E32p.read(r) for r in range(len(Ns))]
    E32p.close()
    # FP64, batched
    E64 = sh.Ensemble(ctx, sh.FAMILY_AXION_LAP1, sh.PREC_FP64, Ns, [dx] * len(Ns), params)
    for r, st in enumerate(states):
        E64.write(r, st)
    E64.set_time(e["eta0"])
    E64.tune(dt)
    E64.set_graph(True)
    ms64b = timed(lambda: E64.step(dt, 1))
    E64.close()
    # FP64 plain: one drop-in level per realisation
    levels = []
    for r, (N, st) in enumerate(zip(Ns, states)):
        lv = sh.Level.periodic(ctx, "AxionStringsLap1", N, 1)
        lv.write(st)
        lv.set_time(e["eta0"])
        levels.append(lv)

    def plain_step():
        for r, lv in enumerate(levels):
            lv.advance(sh.RKN4, dt, dx, params=[float(lam[r]), 0.0])

    ms64 = timed(plain_step)
    # reference values at the end from the plain FP64 run
    E = sh.Ensemble(ctx, sh.FAMILY_AXION_LAP1, sh.PREC_FP64, Ns, [dx] * len(Ns), params)
    f64 = []
    for r, lv in enumerate(levels):
        f = lv.read()
        f64.append(f)
        E.write(r, f)
        lv.close()
    E.set_time(e["eta0"] + total * dt)
    e64 = E.energy()
    s64 = E.string_count()
    E.close()
    rel_l2 = [float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(f32, f64)]
    rel_l2p = [float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(f32p, f64)]
    rel_e = np.abs(e32 - e64) / np.abs(e64)
    big = s64 >= 100
    rel_s = np.abs(s32 - s64)[big] / s64[big]
    tot_s = abs(float(s32.sum() - s64.sum())) / float(s64.sum())
    cu = cells * steps
    out = {
        "workload": f"{e['nreal']} axion-string realisations, N in {list(e['sizes'])} "
                    f"(seeded), lambda log-uniform {list(e['lam'])}, 7-point Laplacian, RKN4, "
                    f"dx {dx}, dt {dt}, eta0 {e['eta0']}, {total} steps",
        "cells": cells, "timed_steps": steps,
        "fp32_kahan_batched": {"value": cu / (ms32 / 1e3), "ms_per_step": ms32 / steps,
                               "tile_nz": nz, "plane_staging": staging32, "graph": True,
                               "gpu_launches_per_step": launches32 / (warmup + steps),
                               "device_bytes": info32["device_bytes"],
                               "wall_s_incl_upload": wall32},
        "fp32_plain_batched": {"value": cu / (ms32p / 1e3), "ms_per_step": ms32p / steps,
                               "field_rel_l2_max": float(max(rel_l2p)),
                               "field_rel_l2_median": float(np.median(rel_l2p)),
                               "string_count_total_rel": abs(float(s32p.sum() - s64.sum())) /
                               float(s64.sum())},
        "fp64_batched": {"value": cu / (ms64b / 1e3), "ms_per_step": ms64b / steps},
        "fp64_plain": {"value": cu / (ms64 / 1e3), "ms_per_step": ms64 / steps,
                       "note": "one sh_level per realisation, sh_level_advance in turn"},
        "speedup_fp32_batched_vs_fp64_plain": ms64 / ms32,
        "error_vs_fp64": {
            "at_step": total,
            "string_count_total_rel": tot_s,
            "string_count_rel_max": float(rel_s.max()) if rel_s.size else None,
            "string_count_rel_median": float(np.median(rel_s)) if rel_s.size else None,
            "realisations_with_100plus_string_cells": int(big.sum()),
            "energy_rel_max": float(rel_e.max()),
            "field_rel_l2_max": float(max(rel_l2)),
            "field_rel_l2_median": float(np.median(rel_l2)),
        },
    }
    return out


FOPT = dict(N=384, dx=0.25, dt=0.05, lambda_bar=0.8, nbubbles=64, t_nuc=(0.0, 20.0),
            t_end=25.0, radius=6.0, width=1.0, amplitude=1.0, inv_dx=8.0, seed=0,
            max_grid=128)


def lambda_bar_params(lambda_bar):
    """FirstOrderPhaseTransition's pure lambda-bar potential
    (FirstOrderPhaseTransition.cpp:19-24): q2 = -1, q3 = 3 n / (4 lb),
    q4 = -n^2 / (8 lb), n = 3 + sqrt(9 - 8 lb); false vacuum 0, true vacuum
    1 for lb < 9/8."""
    n = 3.0 + np.sqrt(9.0 - 8.0 * lambda_bar)
    return [-1.0, 3.0 * n / (4.0 * lambda_bar), -n * n / (8.0 * lambda_bar)]


def fopt_bubbles():
    """Seeded bubble centres and nucleation times (sorted) and the tanh wall
    profile phi = A/2 (1 - tanh((r - R)/w)), dphi = 0."""
    f = FOPT
    rng = np.random.default_rng(f["seed"])
    L = f["N"] * f["dx"]
    xyz = rng.uniform(0.0, L, size=(f["nbubbles"], 3))
    tn = np.sort(rng.uniform(f["t_nuc"][0], f["t_nuc"][1], f["nbubbles"]))
    Lcut = f["radius"] + 8.0 * f["width"]
    nbins = int(Lcut * f["inv_dx"]) + 2
    r = np.arange(nbins) / f["inv_dx"]
    prof = np.stack([0.5 * f["amplitude"] * (1.0 - np.tanh((r - f["radius"]) / f["width"])),
                     np.zeros(nbins)])
    return xyz, tn, prof, Lcut


def spectrum_times(call):
    """Time-to-spectrum in ms (host clock around the synchronous call, bins
    on the host at the end): the first (cold) call of each kind builds its
    bin lists and FFT plan; warm is the median of three calls after both
    kinds were built, alternating binned and unbinned.  Returns the times
    and the (binned, unbinned) spectra."""
    out, spec = {}, {}
    for ub in (False, True):
        t0 = time.perf_counter()
        spec[ub] = call(ub)[0]
        out["unbinned_cold" if ub else "binned_cold"] = 1e3 * (time.perf_counter() - t0)
    warm = {False: [], True: []}
    for _ in range(3):
        for ub in (False, True):
            t0 = time.perf_counter()
            call(ub)
            warm[ub].append(1e3 * (time.perf_counter() - t0))
    out["binned_warm"] = float(np.median(warm[False]))
    out["unbinned_warm"] = float(np.median(warm[True]))
    return out, (spec[False], spec[True])


def run_fopt_leg(sh, ctx, stream, flush, steps, warmup):
    """First-order phase transition with GW tensor, 384^3 periodic, leapfrog,
    64 bubbles injected at their nucleation times (at the first step whose
    time has passed it, as FindBubbles does): FP32+Kahan ensemble path
    against the FP64 plain path (drop-in level with the project's hooks).
    Both run to t_end; steps [warmup, warmup + steps) are timed.  Errors at
    t_end: fields, FP64 energy, GW spectrum (per bin and total)."""
    import torch
    f = FOPT
    N, dx, dt = f["N"], f["dx"], f["dt"]
    nsteps = int(round(f["t_end"] / dt))
    xyz, tn, prof, Lcut = fopt_bubbles()
    q = lambda_bar_params(f["lambda_bar"])
    state0 = np.zeros((14, N, N, N))

    def run(obj_step, inject, t_of):
        nxt = 0
        ev = []
        for s in range(nsteps):
            t = s * dt
            due = []
            while nxt < len(tn) and tn[nxt] <= t:
                due.append(nxt)
                nxt += 1
            timed = warmup <= s < warmup + steps
            if timed:
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
            if due:
                inject(xyz[due])
            obj_step()
            if timed:
                b.record(stream)
                ev.append((a, b))
        torch.cuda.synchronize()
        return float(sum(a.elapsed_time(b) for a, b in ev))

    out = {}
    # FP32 + Kahan (ensemble path, one realisation, graph steps)
    E = sh.Ensemble(ctx, sh.FAMILY_FOPT_GW, sh.PREC_FP32_KAHAN, [N], [dx], [*q, 0.0])
    E.write(0, state0)
    E.set_time(0.0)
    E.set_graph(True)
    ms32 = run(lambda: E.step(dt, 1),
               lambda c: E.add_bubbles(0, c, prof, f["inv_dx"], Lcut), None)
    e32 = E.energy()[0]
    spec32_ms, (gw32, gu32) = spectrum_times(lambda ub: E.gw_spectrum(
        0, zero_padding=1, projection_type=2, unbinned=ub))
    # the same spectra with FP32 transforms and projection (FP64 bin sums)
    E.set_spectrum_precision(sh.PREC_FP32)
    spec32f_ms, (gw32f, gu32f) = spectrum_times(lambda ub: E.gw_spectrum(
        0, zero_padding=1, projection_type=2, unbinned=ub))
    f32 = E.read(0)
    t32 = E.time()
    E.close()
    # FP64 plain path
    lv = sh.Level.periodic(ctx, "FirstOrderPhaseTransition", N, 2, max_grid=f["max_grid"],
                           with_gw=True)
    lv.write(state0)
    lv.set_time(0.0)
    params = [0.0, *q, 0.0, 0.0, 0.0]
    ms64 = run(lambda: lv.advance(sh.LEAPFROG, dt, dx, params=params),
               lambda c: lv.add_bubbles(c, prof, f["inv_dx"], Lcut, dx), None)
    spec64_ms, (gw64, gu64) = spectrum_times(lambda ub: lv.gw_spectrum(
        zero_padding=1, projection_type=2, unbinned=ub))
    f64 = lv.read()
    t64 = lv.time()[0]
    lv.close()
    E = sh.Ensemble(ctx, sh.FAMILY_FOPT_GW, sh.PREC_FP64, [N], [dx], [*q, 0.0])
    E.write(0, f64)
    E.set_time(nsteps * dt)
    e64 = E.energy()[0]
    E.close()
    cu = N ** 3 * steps

    def spec_err(a, b):
        sig = b > 1e-6 * b.max()
        rel = np.abs(a - b)[sig] / b[sig]
        return {"total_rel": float(abs(a.sum() - b.sum()) / b.sum()),
                "bin_rel_max": float(rel.max()) if rel.size else None,
                "bin_rel_median": float(np.median(rel)) if rel.size else None,
                "bins_compared": int(sig.sum()), "bins": int(b.size)}

    out = {
        "workload": f"FOPT + GW tensor {N}^3 periodic, dx {dx}, dt {dt}, leapfrog, 4th-order "
                    f"stencils, lambda-bar potential (lambda_bar {f['lambda_bar']}: q2,q3,q4 = "
                    f"{[round(x, 6) for x in q]}), "
                    f"{f['nbubbles']} tanh bubbles (R {f['radius']}, w {f['width']}, A "
                    f"{f['amplitude']}) nucleated uniformly in t {list(f['t_nuc'])}, "
                    f"{nsteps} steps to t {f['t_end']}",
        "timed_steps": steps,
        "fp32_kahan": {"value": cu / (ms32 / 1e3), "ms_per_step": ms32 / steps,
                       "gw_spectrum_ms": spec32_ms,
                       "gw_spectrum_fp32_transforms_ms": spec32f_ms},
        "fp64_plain": {"value": cu / (ms64 / 1e3), "ms_per_step": ms64 / steps,
                       "gw_spectrum_ms": spec64_ms,
                       "note": f"drop-in level, boxes of {f['max_grid']}^3"},
        "speedup_fp32_vs_fp64_plain": ms64 / ms32,
        "error_vs_fp64": {
            "at_t": nsteps * dt,
            "phi_rel_l2": float(np.linalg.norm(f32[0] - f64[0]) / np.linalg.norm(f64[0])),
            "u_rel_l2": float(np.linalg.norm(f32[2:8] - f64[2:8]) / np.linalg.norm(f64[2:8])),
            "energy_rel": float(abs(e32 - e64) / abs(e64)),
            "time_abs": float(abs(t32 - t64)),
            "gw_binned": spec_err(gw32, gw64),
            "gw_unbinned": spec_err(gu32, gu64),
            "gw_binned_fp32_transforms": spec_err(gw32f, gw64),
            "gw_unbinned_fp32_transforms": spec_err(gu32f, gu64),
        },
    }
    return out


SERVE = dict(nreq=16, rate=4.0, d=(8.0, 40.0), gamma=(1.0, 4.0), lambda_bar=(0.6, 1.0),
             sizes=(64, 96, 128, 192, 256), max_n=128, radius=4.0, width=1.0, cfl=0.2,
             inv_dx=16.0, seed=11, levels=(0, 1, 2), min_base=32, te_crit=1e-2,
             regrid_steps=8)


def serve_requests(max_n, amr=False):
    """Two-bubble collisions (seeded): separation d, wall Lorentz factor
    gamma (radial tanh wall of width w/gamma moving outwards at v), thick or
    thin wall (lambda_bar), Poisson arrivals; box L = d + 2R + 16 with the
    smallest N of the size set that puts 1.5 cells across the contracted
    wall, at most max_n; run to t = 2d.  With amr, each request draws 0, 1
    or 2 refinement levels (from a stream of its own, so the requests are
    otherwise the same): with m levels the base grid has N / 2^m cells per
    side (at least min_base), the finest level has the single-level
    request's resolution where the truncation errors of Phi and dPhi exceed
    te_crit (relative to their maxima, as FirstOrderPhaseTransition's
    TruncationModifier scales them), and the grids are remade every
    regrid_steps coarse steps."""
    sv = SERVE
    rng = np.random.default_rng(sv["seed"])
    rng_levels = np.random.default_rng(sv["seed"] + 1)
    arr = np.cumsum(rng.exponential(1.0 / sv["rate"], sv["nreq"]))
    out = []
    for q in range(sv["nreq"]):
        d = rng.uniform(*sv["d"])
        gamma = rng.uniform(*sv["gamma"])
        lb = sv["lambda_bar"][int(rng.integers(0, 2))]
        L = d + 2 * sv["radius"] + 16.0
        wc = sv["width"] / gamma
        N = next((n for n in sv["sizes"] if n <= max_n and L / n <= wc / 1.5),
                 max(n for n in sv["sizes"] if n <= max_n))
        dx = L / N
        v = np.sqrt(1.0 - 1.0 / gamma ** 2)
        Lcut = sv["radius"] + 10.0 * wc
        nb = int(Lcut * sv["inv_dx"]) + 2
        r = np.arange(nb) / sv["inv_dx"]
        x = (r - sv["radius"]) / wc
        prof = np.stack([0.5 * (1 - np.tanh(x)), 0.5 * v / wc / np.cosh(x) ** 2])
        c = np.array([[L / 2 - d / 2, L / 2, L / 2], [L / 2 + d / 2, L / 2, L / 2]])
        m = int(sv["levels"][int(rng_levels.integers(0, len(sv["levels"])))]) if amr else 0
        while m > 0 and N >> m < sv["min_base"]:
            m -= 1
        Nb = N >> m
        dxb = L / Nb
        out.append(dict(arrival=float(arr[q]), N=Nb, dx=dxb, dt=sv["cfl"] * dxb, t_end=2 * d,
                        params=[*lambda_bar_params(lb), 0.0], centres=c, profile=prof,
                        inv_dx=sv["inv_dx"], Lcut=Lcut, d=d, gamma=gamma, lambda_bar=lb,
                        max_level=m, te_crit=(sv["te_crit"], sv["te_crit"]),
                        regrid_dt=sv["regrid_steps"] * sv["cfl"] * dxb))
    return out


def run_serve_leg(sh, ctx, max_n):
    """The serving loop on a Poisson trace, FP32+Kahan against FP64 pools:
    p50/p99 time-to-spectrum (submission to spectrum ready, host clock) and
    aggregate cell-updates/s over the busy period; per-request spectrum
    error of FP32 against FP64."""
    def trace(prec, reqs):
        S = sh.Server(ctx, prec)
        t0 = time.perf_counter()
        ids = [None] * len(reqs)
        while True:
            now = time.perf_counter() - t0
            for q, rq in enumerate(reqs):
                if ids[q] is None and rq["arrival"] <= now:
                    ids[q] = S.submit(rq["N"], rq["dx"], rq["dt"], rq["t_end"], rq["params"],
                                      rq["centres"], rq["profile"], rq["inv_dx"], rq["Lcut"],
                                      max_level=rq["max_level"], te_crit=rq["te_crit"],
                                      regrid_dt=rq["regrid_dt"])
            running, queued, _ = S.step()
            if all(i is not None for i in ids) and running == 0 and queued == 0:
                break
            if running == 0 and queued == 0:
                nxt = min(rq["arrival"] for q, rq in enumerate(reqs) if ids[q] is None)
                time.sleep(max(0.0, min(0.05, nxt - (time.perf_counter() - t0))))
        lat, first, last = [], None, 0.0
        for i in ids:
            st, t = S.status(i)
            assert st == 2, f"request {i} state {st}"
            lat.append(t[2] - t[0])
            first = t[0] if first is None else min(first, t[0])
            last = max(last, t[2])
        info = S.info()
        spectra = [S.result(i)[0] for i in ids]
        S.close()
        by_levels = {}
        for m in sorted(set(rq["max_level"] for rq in reqs)):
            lm = [x for x, rq in zip(lat, reqs) if rq["max_level"] == m]
            by_levels[str(m)] = {"requests": len(lm), "p50_s": float(np.percentile(lm, 50)),
                                 "p99_s": float(np.percentile(lm, 99))}
        return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                "max_s": float(max(lat)),
                "cell_updates_per_s": info["cell_updates"] / (last - first),
                "busy_s": last - first, "iterations": info["iterations"],
                "by_refinement_levels": by_levels}, spectra

    reqs = serve_requests(max_n)
    r32, s32 = trace(sh.PREC_FP32_KAHAN, reqs)
    r64, s64 = trace(sh.PREC_FP64, reqs)
    tot = [abs(a.sum() - b.sum()) / b.sum() for a, b in zip(s32, s64)]
    Ns = [rq["N"] for rq in reqs]
    # the same requests with 0-2 refinement levels: an FP32 server (FP32 +
    # Kahan hierarchies for the refined requests) against an FP64 one
    reqs_amr = serve_requests(max_n, amr=True)
    r_amr, sa32 = trace(sh.PREC_FP32_KAHAN, reqs_amr)
    r_amr64, sa64 = trace(sh.PREC_FP64, reqs_amr)
    tot_amr = [abs(a.sum() - b.sum()) / b.sum() for a, b in zip(sa32, sa64)]
    levels = [rq["max_level"] for rq in reqs_amr]
    return {
        "workload": f"{len(reqs)} two-bubble requests, Poisson arrivals {SERVE['rate']}/s "
                    f"(seed {SERVE['seed']}), d ~ U{list(SERVE['d'])}, wall gamma ~ "
                    f"U{list(SERVE['gamma'])}, lambda_bar in {list(SERVE['lambda_bar'])}, "
                    f"N in {sorted(set(Ns))} (cap {max_n}), run to t = 2d, GW spectrum "
                    f"(binned, projection 2) at the end",
        "fp32_kahan": r32, "fp64": r64,
        "with_refinement": {
            "workload": f"the same requests with {levels.count(0)} / {levels.count(1)} / "
                        f"{levels.count(2)} of them at 0 / 1 / 2 refinement levels (base grid "
                        f"N / 2^levels, at least {SERVE['min_base']}; AMR requests as "
                        f"hierarchies of the server's precision, te_crit {SERVE['te_crit']}, "
                        f"regrid every {SERVE['regrid_steps']} coarse steps; spectrum of "
                        f"level 0)",
            "fp32_kahan": r_amr, "fp64": r_amr64,
            "gw_total_rel_err_fp32_vs_fp64": {
                "max": float(max(tot_amr)), "median": float(np.median(tot_amr)),
                "by_refinement_levels": {
                    str(m): float(max(t for t, rq in zip(tot_amr, reqs_amr)
                                      if rq["max_level"] == m))
                    for m in sorted(set(levels))}}},
        "gw_total_rel_err_fp32_vs_fp64": {"max": float(max(tot)),
                                          "median": float(np.median(tot))},
    }


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *e):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        smax = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for s in self.samples for q in range(4)
                          if len(s) > 3 + q and s[3 + q].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(self.samples)}


def amr_config(sh, precision=0):
    a = AMR
    return sh.amr_config(a["project"], precision=precision, N0=a["N0"], L=a["L"], cfl=a["cfl"],
                         t_start=a["t_start"],
                         nghost=a["nghost"], max_level=a["max_level"],
                         blocking_factor=a["blocking_factor"], max_grid_size=a["max_grid_size"],
                         n_error_buf=a["n_error_buf"], regrid_dt=a["regrid_dt"],
                         te_crit=[a["te_crit"]] * 4, params=a["params"],
                         string_width_threshold=a["string_width_threshold"],
                         max_local_regrids=a["max_local_regrids"])


def amr_state():
    return load_ic().axion_string_ic(AMR["N0"], AMR["L"], kmax=1.0, seed=0)


def single_state():
    s = SINGLE
    return load_ic().axion_string_ic(s["N"], s["L"], kmax=1.0, seed=s["seed"])


def single_config():
    """The headline workload's config; both arms print exactly this dict."""
    s = SINGLE
    dx = s["L"] / s["N"]
    return {"workload": "axion strings 128^3 periodic single level, L=32, 7-point Laplacian, "
                        "lambda=1, RKN4, eta0=0.1, dt=0.25 dx, FP64 (200-step job)",
            "N": s["N"], "L": s["L"], "dx": dx, "dt": 0.25 * dx, "eta0": s["eta0"],
            "job_steps": s["total_steps"], "project": s["project"],
            "integrator": "RKN4 (type 21)", "ic": "seeded Gaussian field, |k|<=1, seed 0",
            "l2": "flushed between timed steps (512 MB write, outside events)"}


def amr_leg_config():
    a = AMR
    return {"workload": "axion strings AMR: 256^3 coarse + 2 refinement levels (ratio 2, "
                        "blocking factor 8, max grid 32), 4th-order Laplacian, lambda=1, "
                        "RKN4 with subcycling, winding + truncation-error tags "
                        "(te_crit 1e-3), FP64; timed coarse steps all hold 3 levels",
            "N0": a["N0"], "L": a["L"], "dx0": a["L"] / a["N0"], "cfl": a["cfl"],
            "eta0": a["t_start"], "eta_end": a["t_end"],
            "string_width_threshold": a["string_width_threshold"],
            "regrid_dt": a["regrid_dt"], "n_error_buf": a["n_error_buf"],
            "regrids": "global (amr.max_local_regrids = 0)",
            "project": a["project"], "integrator": "RKN4 (type 21)",
            "l2": "flushed between timed steps (512 MB write, outside events)"}


def host_cores():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def cpu_baseline_single(budget_s=12.0, max_steps=400):
    """The oracle on the host cores: RKN4 steps of the 128^3 level until
    about budget_s seconds."""
    from tests.oracle_lib import Oracle
    s = SINGLE
    dx = s["L"] / s["N"]
    orc = Oracle()
    st = single_state()
    steps, el, batch = 0, 0.0, 2
    while el < budget_s and steps < max_steps:
        t0 = time.perf_counter()
        st = orc.evolve_periodic(s["project"], 21, st, t0=s["eta0"] + steps * 0.25 * dx,
                                 dt=0.25 * dx, dx=dx, nsteps=batch, params=s["params"],
                                 nghost=s["nghost"])
        el += time.perf_counter() - t0
        steps += batch
        batch = min(2 * batch, 64)
    return {"value": s["N"] ** 3 * steps / el, "unit": METRIC, "cores": host_cores(),
            "kind": "port",
            "sample": f"{steps} RKN4 steps of the 128^3 level (oracle, FP64, OpenMP), {el:.1f} s"}


def run_reference(args):
    """The reference's CPU implementation of the path (oracle port) on the
    host cores, on the headline workload: W warm-up RKN4 steps of the 128^3
    level, then the K timed steps in one call, so that the level stays in
    the oracle's memory between steps as it would in the reference's own
    loop (one step per call would time the host-side copies in and out of
    the oracle instead).  Only the oracle library and numpy are loaded."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from tests.oracle_lib import Oracle
    s = SINGLE
    dx = s["L"] / s["N"]
    dt = 0.25 * dx
    orc = Oracle()
    st = single_state()
    st = orc.evolve_periodic(s["project"], 21, st, t0=s["eta0"], dt=dt, dx=dx,
                             nsteps=args.warmup, params=s["params"], nghost=s["nghost"])
    t0 = time.perf_counter()
    st = orc.evolve_periodic(s["project"], 21, st, t0=s["eta0"] + args.warmup * dt, dt=dt,
                             dx=dx, nsteps=args.steps, params=s["params"], nghost=s["nghost"])
    el = time.perf_counter() - t0
    value = float(s["N"] ** 3 * args.steps / el)
    cores = host_cores()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Gaussian random field, |k|<=1)",
        "config": single_config(),
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} RKN4 steps of the 128^3 level in one call of "
                                   f"the oracle port, {cores} threads (reference build "
                                   f"unavailable: AMReX absent)"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def replica_aggregate(total_ms, cell_updates, world, device):
    """Whole-job throughput of `world` independent replicas (one per rank):
    the cell-updates of all ranks over the slowest rank's timed region.
    Returns (cell-updates/s, max time in ms)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([total_ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        c = torch.tensor([float(cell_updates)], dtype=torch.float64, device=device)
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
        total_ms, cell_updates = float(t.item()), float(c.item())
    return cell_updates / (total_ms / 1e3), total_ms


def run_case(name):
    """Small fixed cases for profiler captures (no timing, no output line):
    axion-fp32k / axion-fp32k-tma / axion-fp64: one 256^3 axion
    realisation, 3 RKN4 steps (9 stage launches; -tma with the stencil planes
    staged by tensor copies); fopt-fp32k: one 192^3 FOPT + GW realisation, 3
    leapfrog steps; gw384 / gw256: GW spectra of an FP64 FOPT + GW level
    (binned and unbinned, twice each); amr / amr128 / amr-fp32: the AMR
    workload at N0 = 64 (L = 16) or N0 = 128 (L = 32), 60 coarse steps (three
    levels at the end), or at N0 = 64 on FP32 + Kahan levels; single: the 128^3
    FP64 level, 3 RKN4 steps; fp64-peak: prints the measured FP64 FMA issue
    rate (the FP64 roofline's peak)."""
    import sledgehamr_gb300 as sh
    from sledgehamr_gb300 import ic
    if name == "fp64-peak":
        r = fp64_probe(0)
        print(json.dumps({"fp64_fma_per_s": r, "fp64_tflops": 2 * r / 1e12 if r else None}))
        return
    ctx = sh.Context(0)
    if name.startswith("axion"):
        prec = sh.PREC_FP64 if name.endswith("fp64") else sh.PREC_FP32_KAHAN
        N = 256
        E = sh.Ensemble(ctx, sh.FAMILY_AXION_LAP1, prec, [N], [0.25], [1, 0, 0, 0])
        E.write(0, ic.axion_string_ic(N, N * 0.25, kmax=1.0, seed=0))
        E.set_time(0.1)
        if name.endswith("tma"):
            E.set_staging(1)
        E.step(0.0625, 3)
        E.close()
    elif name == "fopt-fp32k":
        N = 192
        q = lambda_bar_params(0.8)
        E = sh.Ensemble(ctx, sh.FAMILY_FOPT_GW, sh.PREC_FP32_KAHAN, [N], [0.25], [*q, 0.0])
        st = np.zeros((14, N, N, N))
        st[0] = 0.5 + 0.2 * ic.gaussian_field(N, N * 0.25, 2.0, 1)
        E.write(0, st)
        E.step(0.05, 3)
        E.close()
    elif name in ("amr", "amr128", "amr-fp32"):
        a = AMR
        n0 = 128 if name == "amr128" else 64
        prec = sh.PREC_FP32_KAHAN if name == "amr-fp32" else sh.PREC_FP64
        cfg = sh.amr_config(a["project"], precision=prec, N0=n0, L=n0 * 0.25, cfl=a["cfl"],
                            t_start=a["t_start"],
                            nghost=a["nghost"], max_level=a["max_level"],
                            blocking_factor=a["blocking_factor"],
                            max_grid_size=a["max_grid_size"], n_error_buf=a["n_error_buf"],
                            regrid_dt=a["regrid_dt"], te_crit=[a["te_crit"]] * 4,
                            params=a["params"],
                            string_width_threshold=a["string_width_threshold"])
        sim = sh.Amr(ctx, cfg, ic.axion_string_ic(n0, n0 * 0.25, kmax=1.0, seed=0))
        for q in range(60):
            sim.step(1)
            # valid cells and stage-kernel tiles (grid size) of every level,
            # to relate a profiled launch to the cells it updated
            rows = []
            for lev in range(sim.info()["finest"] + 1):
                v = sim.level(lev)
                tiles = 0
                for lo, hi in v.boxes:
                    nx_, ny_, nz_ = (hi[0] - lo[0] + 1, hi[1] - lo[1] + 1, hi[2] - lo[2] + 1)
                    for x0 in range(0, nx_, 32):
                        w = min(32, nx_ - x0)
                        tiles += -(-nz_ // 8) * -(-ny_ // (128 // w))
                rows.append((lev, v.nvalid, tiles))
            print("step", q, rows, flush=True)
        sim.close()
    elif name in ("gw384", "gw256"):
        # the GW spectrum of a 384^3 (256^3) FOPT + GW level (FP64, binned
        # and unbinned, each twice: the second call of each kind is warm)
        N = int(name[2:])
        lv = sh.Level.periodic(ctx, "FirstOrderPhaseTransition", N, 2, max_grid=128,
                               with_gw=True)
        st = np.zeros((14, N, N, N))
        for q in range(6):
            st[8 + q] = 1e-3 * ic.gaussian_field(N, N * 0.25, 2.0, 40 + q)
        lv.write(st)
        del st
        for ub in (False, True, False, True):
            t0 = time.perf_counter()
            lv.gw_spectrum(zero_padding=1, projection_type=2, unbinned=ub)
            print("gw spectrum", "unbinned" if ub else "binned",
                  f"{1e3 * (time.perf_counter() - t0):.1f} ms", flush=True)
        lv.close()
    elif name == "single":
        s = SINGLE
        lv = sh.Level.periodic(ctx, s["project"], s["N"], s["nghost"])
        lv.write(single_state())
        lv.set_time(s["eta0"])
        dx = s["L"] / s["N"]
        for _ in range(3):
            lv.advance(sh.RKN4, 0.25 * dx, dx, params=s["params"])
        lv.close()
    else:
        raise SystemExit(f"unknown case {name}")
    ctx.synchronize()
    ctx.close()


def timed_steps(step, steps, warmup, stream, flush, clk=None, before=None):
    """W untimed steps, then K steps each bracketed by CUDA events on the
    library's stream with an L2 flush outside the events; returns the summed
    milliseconds (and the per-step values of `before`, called before each
    timed step)."""
    import torch
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    seen = []
    for q in range(steps):
        flush.zero_()
        if before is not None:
            seen.append(before())
        starts[q].record(stream)
        step()
        ends[q].record(stream)
    torch.cuda.synchronize()
    return float(sum(a.elapsed_time(b) for a, b in zip(starts, ends))), seen


# FP64 thread instructions (DFMA + DMUL + DADD) per cell-update of the stage
# kernels (ncu executed-instruction counters of the three launches of one RKN4
# step divided by the cells): the 7-point kernel of the 128^3 level
# (`--case single`) and the 13-point kernel of the AMR workload (level 0 of
# `--case amr`; the per-cell count does not depend on the level).
FP64_INSTR_PER_CELL_UPDATE = {"single": 55.25, "amr": 61.625}


def fp64_probe(device):
    """Measured FP64 FMA issue rate of the GPU (thread instructions/s)."""
    import ctypes as C
    from sledgehamr_gb300 import _lib
    r = C.c_double()
    rc = _lib.load().sh_probe_fp64_fma_rate(device, C.byref(r))
    return r.value if rc == 0 else None


def fp64_roofline(roof, workload, device):
    """The stage kernels' FP64 instruction issue over their duration against
    the measured FP64 FMA rate."""
    per = FP64_INSTR_PER_CELL_UPDATE.get(workload)
    peak = fp64_probe(device)
    out = {"bound": "fp64", "unit": "FP64 thread instructions/s", "peak": peak,
           "peak_kind": "measured (sh_probe_fp64_fma_rate: dependent DFMA chains, all SMs)",
           "instructions_per_cell_update": per}
    if per and peak and roof.get("stage_ms_total"):
        cu = roof["_cell_updates"]
        ach = per * cu / (roof["stage_ms_total"] / 1e3)
        out.update({"achieved": ach, "frac": ach / peak})
    return out


def stage_roofline(ctx, words, cell_updates, traffic_b, peak, peak_kind):
    """HBM roofline of the stage kernels from the library's per-launch CUDA
    events (profile category "rhs") over the timed region."""
    stage_ms, stage_launches = ctx.profile_read("rhs")
    fill_ms, fill_launches = ctx.profile_read("fill_patch")
    other = {c: ctx.profile_read(c)[0] for c in ("coarse_fine", "average_down", "tagging",
                                                  "data_move")}
    achieved = words * 8 * cell_updates / (stage_ms / 1e3) / 1e9
    cells_per_launch = 3.0 * cell_updates / max(stage_launches, 1)
    traffic = traffic_b / 3.0 * cells_per_launch if traffic_b else None
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
            "algorithmic_bytes_per_launch": words * 8 / 3.0 * cells_per_launch,
            "kernel": "stage_kernel (fused Rhs + RKN4 stage update)",
            "bytes_per_cell_update": words * 8, "stage_ms_total": stage_ms,
            "stage_launches": stage_launches, "stage_ms_per_launch":
            stage_ms / max(stage_launches, 1), "fill_ms_total": fill_ms,
            "fill_launches": fill_launches, "other_ms": other, "_cell_updates": cell_updates}


def run_amr_leg(sh, ctx, stream, flush, steps, warmup, peak, peak_kind):
    """The AMR workload with every level present in the timed window: coarse
    steps (untimed) until the hierarchy reaches max_level, W more warm-up
    steps, then K timed coarse steps (at most up to eta_end).  e2e: the same
    job (from the host initial state to the end of the timed window) through
    the C ABI with the final hierarchy read back to pinned host memory."""
    import torch
    a = AMR
    dt0 = a["cfl"] * a["L"] / a["N0"]
    job = int(np.ceil((a["t_end"] - a["t_start"]) / dt0 - 1e-9))
    state = amr_state()
    sim = sh.Amr(ctx, amr_config(sh), state)
    pre = 0
    while sim.info()["finest"] < a["max_level"] and pre < job:
        sim.step(1)
        pre += 1
    for _ in range(warmup):
        sim.step(1)
        pre += 1
    K = max(1, min(steps, job - pre))
    l0 = ctx.kernel_launches
    cu0 = sim.info()["cell_updates"]
    tm0 = sim.timers()
    ctx.profile(True)
    ms, finest = timed_steps(lambda: sim.step(1), K, 0, stream, flush,
                             before=lambda: sim.info()["finest"])
    launches = ctx.kernel_launches - l0
    cus = sim.info()["cell_updates"] - cu0
    roof = stage_roofline(ctx, WORDS_PER_CELL_UPDATE, cus, TRAFFIC_B_PER_CELL_UPDATE["amr"],
                          peak, peak_kind)
    ctx.profile(False)
    roof["fp64_roofline"] = fp64_roofline(roof, "amr", torch.cuda.current_device())
    roof.pop("_cell_updates", None)
    info = sim.info()
    levels = [{"level": l, "boxes": sim.level(l).nbox, "cells": sim.level(l).nvalid}
              for l in range(info["finest"] + 1)]
    timers = window_timers(sim, tm0)
    # the precision form on the same hierarchy: FP32 + Kahan levels, FP64
    # truncation errors and tags, the same pre-roll and timed window
    fp32 = run_amr_fp32(sh, ctx, stream, flush, K, pre, sim, ms)
    sim.close()
    # e2e: the same job from pinned host memory, read back at the end
    host_in = torch.from_numpy(np.ascontiguousarray(state)).pin_memory()
    host_levels = [torch.empty(lv_["cells"] * 4, dtype=torch.float64).pin_memory()
                   for lv_ in levels]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim2 = sh.Amr(ctx, amr_config(sh), host_in.numpy())
    for _ in range(pre + K):
        sim2.step(1)
    e2e_cus = sim2.info()["cell_updates"]
    d2h = 0
    for l in range(sim2.info()["finest"] + 1):
        v = sim2.level(l)
        n = v.nvalid * v.ncomp
        out = host_levels[l] if (l < len(host_levels) and host_levels[l].numel() == n) else \
            torch.empty(n, dtype=torch.float64).pin_memory()
        ctx.check(ctx.lib.sh_level_read(ctx.h, v.h, sh.SH_NEW, 1, out.data_ptr()), "read")
        d2h += n * 8
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    sim2.close()
    out = {"config": amr_leg_config(), "value": cus / (ms / 1e3), "unit": METRIC,
           "timed_steps": K, "ms_per_step": ms / K, "untimed_steps_before": pre,
           "eta_timed": [a["t_start"] + pre * dt0, a["t_start"] + (pre + K) * dt0],
           "levels_in_timed_window": sorted({f + 1 for f in finest}),
           "gpu_launches_per_step": launches / K,
           "stage_launches_per_step": roof["stage_launches"] / K,
           "cell_updates_timed": cus, "levels_at_end": levels,
           "host_timers_s": timers, "roofline": roof, "fp32_kahan": fp32,
           "e2e": {"value": e2e_cus / e2e_s, "unit": METRIC, "job_steps": pre + K,
                   "h2d_bytes_per_step": state.size * 8 / (pre + K),
                   "d2h_bytes_per_step": d2h / (pre + K),
                   "note": "whole job from the host initial state: the pre-roll to full "
                           "depth and the timed window, hierarchy read back at the end"}}
    return out


def window_timers(sim, before):
    """Host seconds per time-stepper phase spent since `before` (the
    timed window), rounded."""
    return {k: round(v[0] - before.get(k, (0.0, 0))[0], 4) for k, v in sim.timers().items()}


def amr_levels(sh, ctx, sim):
    """Boxes, FP64 values (boxes layout, on the device) and string-tag
    counts of every level of a hierarchy."""
    import torch
    a = AMR
    dt0 = a["cfl"] * a["L"] / a["N0"]
    out = []
    for l in range(sim.info()["finest"] + 1):
        v = sim.level(l)
        d = torch.empty(v.nvalid * v.ncomp, dtype=torch.float64, device="cuda")
        ctx.check(ctx.lib.sh_level_read_device(ctx.h, v.h, sh.SH_NEW, 1, d.data_ptr()), "read")
        t = v.time()[0]
        tags = v.string_tags(t, l, dt0 / 2 ** l, a["L"] / a["N0"] / 2 ** l)
        out.append((v.boxes, d, tags))
    return out


def run_amr_fp32(sh, ctx, stream, flush, K, pre, sim64, ms64):
    """The AMR workload on FP32 + Kahan levels (sh_amr_config.precision):
    the FP64 leg's pre-roll, then its K timed coarse steps; errors at the
    end against the FP64 hierarchy (which has run the same steps): relative
    L2 per level where the boxes agree, and the string-tag counts."""
    import torch
    sim = sh.Amr(ctx, amr_config(sh, sh.PREC_FP32_KAHAN), amr_state())
    for _ in range(pre):
        sim.step(1)
    cu0 = sim.info()["cell_updates"]
    tm0 = sim.timers()
    ctx.profile(True)
    ms, finest = timed_steps(lambda: sim.step(1), K, 0, stream, flush,
                             before=lambda: sim.info()["finest"])
    cus = sim.info()["cell_updates"] - cu0
    stage_ms, stage_n = ctx.profile_read("rhs")
    fill_ms, _ = ctx.profile_read("fill_patch")
    cf_ms, _ = ctx.profile_read("coarse_fine")
    other = {c: ctx.profile_read(c)[0] for c in ("average_down", "tagging", "data_move")}
    ctx.profile(False)
    timers = window_timers(sim, tm0)
    mine, ref = amr_levels(sh, ctx, sim), amr_levels(sh, ctx, sim64)
    err = []
    for l, ((b32, d32, t32), (b64, d64, t64)) in enumerate(zip(mine, ref)):
        row = {"level": l, "boxes_equal": b32 == b64, "string_tags_fp32": t32,
               "string_tags_fp64": t64}
        if b32 == b64:
            row["rel_l2"] = float(torch.linalg.norm(d32 - d64) / torch.linalg.norm(d64))
        err.append(row)
    sim.close()
    del mine, ref
    return {"value": cus / (ms / 1e3), "unit": METRIC, "ms_per_step": ms / K,
            "speedup_vs_fp64": ms64 / ms, "levels_in_timed_window": sorted({f + 1 for f in finest}),
            "stage_ms_total": stage_ms, "stage_launches": stage_n, "fill_ms_total": fill_ms,
            "coarse_fine_ms_total": cf_ms, "other_ms": other, "host_timers_s": timers,
            "error_vs_fp64": err,
            "note": "FP32 values with FP32 Kahan compensations on every level, FP32 stage "
                    "arithmetic (csrc/sh_stage32.cuh), FP32 ghost fills and average-down "
                    "pairs; truncation errors, tags through the project hooks and time in FP64"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--legs", default="amr,ensemble,fopt,serve",
                    help="comma list of the legs reported beside the headline (amr, "
                         "ensemble, fopt, serve; empty for none)")
    ap.add_argument("--serve-max-n", type=int, default=SERVE["max_n"])
    ap.add_argument("--case", default=None,
                    help="run one small profiling case and exit: axion-fp32k, axion-fp64, "
                         "axion-fp32k-tma, fopt-fp32k, amr, amr128, amr-fp32, single, gw384, "
                         "gw256, "
                         "fp64-peak")
    args = ap.parse_args()
    if args.case:
        run_case(args.case)
        return
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import sledgehamr_gb300 as sh

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    ctx = sh.Context(local)
    # one explicit stream for the library's kernels, the CUDA events and the
    # L2 flush (the legacy default stream does not order with the library's
    # own non-blocking stream)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    peak, peak_kind = peaks()

    # ---- headline: the 128^3 level on the drop-in path -------------------
    s = SINGLE
    N = s["N"]
    dx = s["L"] / N
    dt = 0.25 * dx
    state = single_state()
    lv = sh.Level.periodic(ctx, s["project"], N, s["nghost"])
    lv.write(state)
    lv.set_time(s["eta0"])
    for _ in range(args.warmup):
        lv.advance(sh.RKN4, dt, dx, params=s["params"])
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = ctx.kernel_launches
    ctx.profile(True)
    with ClockSampler(local) as clk:
        total_ms, _ = timed_steps(lambda: lv.advance(sh.RKN4, dt, dx, params=s["params"]),
                                  args.steps, 0, stream, flush)
    launches = ctx.kernel_launches - l0
    cus = N ** 3 * args.steps
    roof = stage_roofline(ctx, WORDS_PER_CELL_UPDATE, cus, TRAFFIC_B_PER_CELL_UPDATE["single"],
                          peak, peak_kind)
    ctx.profile(False)
    lv.close()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    value, total_ms = replica_aggregate(total_ms, cus, world, "cuda")
    roof["fp64_roofline"] = fp64_roofline(roof, "single", local)
    roof.pop("_cell_updates", None)

    # e2e: the whole 200-step job through the C ABI with pinned host buffers,
    # the median of three jobs (a job is about 60 ms, so one job's figure
    # moves by a few percent with the host's scheduling)
    host_in = torch.from_numpy(np.ascontiguousarray(state)).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    e2e_runs = []
    for _ in range(E2E_JOBS):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lv2 = sh.Level.periodic(ctx, s["project"], N, s["nghost"])
        ctx.check(ctx.lib.sh_level_write(ctx.h, lv2.h, sh.SH_NEW, 0, host_in.data_ptr()),
                  "write")
        lv2.set_time(s["eta0"])
        for _ in range(s["total_steps"]):
            lv2.advance(sh.RKN4, dt, dx, params=s["params"])
        ctx.check(ctx.lib.sh_level_read(ctx.h, lv2.h, sh.SH_NEW, 0, host_out.data_ptr()),
                  "read")
        torch.cuda.synchronize()
        e2e_runs.append(time.perf_counter() - t0)
        lv2.close()
    e2e_s = float(np.median(e2e_runs))
    e2e = {"value": world * N ** 3 * s["total_steps"] / e2e_s, "unit": METRIC,
           "jobs": E2E_JOBS, "job_s": [round(x, 5) for x in e2e_runs],
           "h2d_bytes_per_step": state.size * 8 / s["total_steps"],
           "d2h_bytes_per_step": state.size * 8 / s["total_steps"],
           "job_steps": s["total_steps"],
           "note": "level created, initial state uploaded from pinned host memory, 200 RKN4 "
                   "steps, final state read back to pinned host memory; median of the jobs"}

    legs = {}
    want = [f for f in args.legs.split(",") if f]
    cpu_ok = rank == 0 and not args.no_cpu_baseline
    if "amr" in want:
        legs["amr"] = run_amr_leg(sh, ctx, stream, flush, args.steps, args.warmup, peak,
                                  peak_kind)
    if "ensemble" in want:
        legs["batched_ensemble"] = run_ensemble_leg(sh, ctx, stream, flush, steps=20,
                                                    warmup=args.warmup)
    if "fopt" in want:
        legs["fopt_precision"] = run_fopt_leg(sh, ctx, stream, flush, steps=20,
                                              warmup=args.warmup)
    if "serve" in want:
        legs["serving"] = run_serve_leg(sh, ctx, args.serve_max_n)
    cpu = cpu_baseline_single() if cpu_ok else None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Gaussian random field, |k|<=1)",
            "config": single_config(), "parallelism": f"replicas x{world}",
            "e2e": e2e, "gpu_launches": launches,
            "gpu_launches_per_step": launches / args.steps,
            "roofline": roof, "clocks": clk.summary(), "cell_updates_timed": cus,
        }
        if cpu:
            line["cpu_baseline"] = cpu
        if legs:
            line["legs"] = legs
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
