"""Benchmark of the time-stepping hot path: cell-updates/s of one GPU.

Workload (one "step" = one RKN4 step, Integrator::Advance, of the level):
  AxionStrings equations, 128^3 periodic single level, L = 32 (dx = 0.25),
  2nd-order (7-point) Laplacian, lambda = 1, eta0 = 0.1, dt = 0.0625, FP64,
  seeded band-limited Gaussian initial state (|k| <= 1, unit variance).
  One cell-update = one valid cell advanced by one full step, all components.

value   : device-resident state; K timed steps, each bracketed by CUDA events
          on the library's stream; L2 flushed (a 512 MB write) between timed
          steps, outside the events.
e2e     : the same step through the public C ABI with host buffers: every
          step uploads the state from pinned host memory, advances, and
          downloads the result (both copies inside the timed region).
roofline: the fused stage kernel, algorithmic bytes per launch divided by its
          average duration, against the measured HBM copy bandwidth.
cpu_baseline: the CPU oracle (FP64 restatement of the reference, OpenMP) on
          the host cores, a bounded sample of the same workload.

--impl reference: the reference's CPU path on the host cores (the oracle
port on this machine; oracle/_ref where the reference could be compiled).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 128
L = 32.0
DX = L / N
DT = 0.25 * DX
ETA0 = 0.1
PROJECT = "AxionStringsLap1"
PARAMS = [1.0, 0.0]
NGHOST = 1
METRIC = "cell-updates/s"
# Algorithmic HBM words per cell-update of the fused RKN4 schedule this
# library runs for 2 position + 2 momentum components (stage i reads the
# stage state, y0 and K_0..K_{i-1} and writes K_i and the next stage state;
# the last stage writes y1): 10 + 16 + 16 = 42 FP64 words.
WORDS_PER_CELL_UPDATE = 42
STAGE_KERNELS_PER_STEP = 3


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


def initial_state():
    from sledgehamr_gb300 import ic
    return ic.axion_string_ic(N, L, kmax=1.0, seed=0)


def cpu_baseline(state, budget_s=12.0, max_steps=400):
    """The oracle on the host cores: RKN4 steps of the full 128^3 level,
    repeated in batches until about budget_s seconds of CPU work."""
    from tests.oracle_lib import Oracle
    orc = Oracle()
    orc.evolve_periodic(PROJECT, 21, state, t0=ETA0, dt=DT, dx=DX, nsteps=1, params=PARAMS,
                        nghost=NGHOST)  # warm-up
    steps, el = 0, 0.0
    batch = 2
    st = state
    while el < budget_s and steps < max_steps:
        t0 = time.perf_counter()
        st = orc.evolve_periodic(PROJECT, 21, st, t0=ETA0 + steps * DT, dt=DT, dx=DX,
                                 nsteps=batch, params=PARAMS, nghost=NGHOST)
        el += time.perf_counter() - t0
        steps += batch
        batch = min(2 * batch, 64)
    return {"value": N ** 3 * steps / el, "unit": METRIC,
            "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
            "kind": "port",
            "sample": f"{steps} RKN4 steps of the 128^3 level (FP64 oracle, OpenMP), {el:.1f} s"}


def run_reference(args):
    """The reference's CPU implementation of the path on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    # The reference's compiled per-cell code (oracle/_ref) has no 7-point
    # Laplacian project, so the workload runs on the oracle port, the FP64
    # restatement of the reference's loop drivers and integrator.
    from tests.oracle_lib import Oracle
    kind = "port"
    orc = Oracle()
    st = initial_state()
    project = PROJECT
    for _ in range(args.warmup):
        orc.evolve_periodic(project, 21, st, t0=ETA0, dt=DT, dx=DX, nsteps=1, params=PARAMS,
                            nghost=NGHOST)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        st = orc.evolve_periodic(project, 21, st, t0=ETA0, dt=DT, dx=DX, nsteps=1,
                                 params=PARAMS, nghost=NGHOST)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * float(np.mean(times))
    value = N ** 3 / (ms / 1e3)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "axion strings 128^3 periodic, RKN4, 7-point Laplacian, FP64",
                   "N": N, "L": L, "dt": DT},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": kind,
                         "sample": f"{args.steps} full RKN4 steps of the 128^3 level"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
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
    # L2 flush (the legacy default stream would not order with the
    # library's own non-blocking stream)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)

    state = initial_state()
    lv = sh.Level.periodic(ctx, PROJECT, N, NGHOST)
    lv.write(state)
    lv.set_time(ETA0)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step():
        lv.advance(sh.RKN4, DT, DX, params=PARAMS)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    l0 = ctx.kernel_launches
    ctx.profile(True)
    with ClockSampler(local) as clk:
        for s in range(args.steps):
            flush.zero_()
            starts[s].record(stream)
            step()
            ends[s].record(stream)
        torch.cuda.synchronize()
    launches = ctx.kernel_launches - l0
    stage_total_ms, stage_launches = ctx.profile_read("rhs")
    fill_total_ms, fill_launches = ctx.profile_read("fill_patch")
    ctx.profile(False)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ms = float(sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / args.steps)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    cells = N ** 3
    value = world * cells / (ms / 1e3)

    # roofline of the fused stage kernel: CUDA events recorded by the library
    # around every stage-kernel launch on its stream during the timed steps
    stage_ms = stage_total_ms / max(stage_launches, 1)
    bytes_per_stage = WORDS_PER_CELL_UPDATE * 8 * cells / STAGE_KERNELS_PER_STEP
    achieved = bytes_per_stage / (stage_ms / 1e3) / 1e9
    peak, peak_kind = peaks()

    # e2e through the public API with pinned host buffers
    host_in = torch.from_numpy(state.astype(np.float64)).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    e2e_steps = max(3, min(args.steps, 10))
    lv.set_time(ETA0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.check(ctx.lib.sh_level_write(ctx.h, lv.h, sh.SH_NEW, 0, host_in.data_ptr()), "write")
        step()
        ctx.check(ctx.lib.sh_level_read(ctx.h, lv.h, sh.SH_NEW, 0, host_out.data_ptr()), "read")
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    nbytes = state.size * 8

    out = np.asarray(host_out.numpy())
    finite = bool(np.isfinite(out).all())
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(state)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Gaussian random field, |k|<=1)",
            "config": {"workload": "axion strings 128^3 periodic single level, RKN4, 7-point "
                                   "Laplacian, lambda=1, FP64", "N": N, "L": L, "dx": DX,
                       "dt": DT, "project": PROJECT, "integrator": "RKN4 (type 21)",
                       "l2": "flushed between timed steps (512 MB write, outside events)",
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": world * cells / e2e_s, "unit": METRIC, "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": nbytes},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None,
                         "peak_kind": peak_kind, "kernel": "stage_kernel (fused Rhs + RKN4 "
                         "stage update)", "bytes_per_launch": bytes_per_stage,
                         "stage_ms": stage_ms, "stage_launches": stage_launches,
                         "ghost_fill_ms": fill_total_ms / max(fill_launches, 1)},
            "clocks": clk.summary(),
            "result_finite": finite,
        }
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    lv.close()
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
