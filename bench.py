#!/usr/bin/env python3
"""Benchmark of the 3dmhd hot path on GB300: cell-RK3-updates/s.

Workload (default): the plain-method FP64 configuration at 512x512x256 with
lMag, lRot (rotation 0.1 about z) and lShr on, polytropic layer with seeded
Gaussian temperature noise, fixed dt = 1e-4.  One "step" is one full Wray RK3
step (three fused substages + wall conditions + ghost fill) over the whole
grid.  The state (about 13 GB) is far larger than L2, so no flush is needed.

  value      interior cells x steps / device time (CUDA events on the
             context's stream), inputs resident in HBM
  e2e        the same metric through the C ABI with pinned HOST buffers:
             every step uploads the state, steps once and downloads it
  roofline   the fused substage kernel: algorithmic HBM bytes per launch over
             its average duration (events around each launch), against the
             measured HBM copy peak; plus the FP64 pipe, which binds first
  cpu_baseline  the CPU oracle (a restatement of the reference's own code,
             bit-exact with it) on a bounded slab of the same workload

`--impl reference` times the reference's CPU implementation of the path
(the oracle port; the reference binary itself cannot be built on the GPU host)
with all host threads on the same metric and configuration.

Multi-GPU (torchrun): replicas only -- every rank steps its own instance;
`value` is the sum over ranks of cells x steps over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "rast-3dmhd-cpp_gb300" / "python"))

from mhd_gb300 import abi  # noqa: E402
from mhd_gb300.case import STATE_FIELDS, config0, config1, config2_batch, config3, initial_state  # noqa: E402

METRIC = "cell-RK3-updates/s"
# Algorithmic HBM traffic of the fused FP64 path per interior cell and RK3
# step: substage 1 reads U and writes U', Z' (24 doubles), substage 2 reads U,
# Z and writes U', Z' (32), substage 3 reads U, Z and writes U' (24) for the
# 8 MHD fields = 640 B; with lShr the persistent FT adds a read and a write
# per substage (48 B).  Hydro-only (5 fields): 400 B.
def algorithmic_bytes_per_cell_step(case) -> float:
    nf = case.nfields
    b = 80.0 * nf
    if case.lShr:
        b += 3 * 16.0
    return b


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        sms, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1", "0x1"):
                    reasons.add(n)
        os.unlink(self.f.name)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sms), "power_w_max": max(power) if power else None}


def measured_peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            pass
    return {}


def case_for(name: str):
    c1 = config1()
    # "mid": the same physics at 256x256x128 (about 1.6 GB of state, larger
    # than L2), the size used for ncu captures
    mid = c1.replace(nPx=256, nPy=256, nPz=128, name="config1_physics_256x256x128")
    return {"config1": c1, "config0": config0(), "mid": mid}[name]


# ---------------------------------------------------------------------------
# CPU baseline (the oracle restating the reference code; checker only)
# ---------------------------------------------------------------------------
def cpu_sample_case(case):
    """A slab of the workload: same horizontal grid and physics, 16 interior
    z planes; the per-cell work of the RK3 step is the same."""
    return case.replace(nPz=16, name=case.name + "_slab16")


ORACLE_FLAGS = "gcc -O2 -std=gnu11 -ffp-contract=off -fno-fast-math -fopenmp"


def _time_oracle_steps(o, n: int, dt: float | None) -> float:
    t = time.perf_counter()
    o.steps(n, dt)
    return time.perf_counter() - t


def cpu_baseline(case, target_s: float = 12.0, threads: int | None = None) -> dict:
    """The reference's algorithm (the oracle) on the host cores, in the two
    run modes of the reference: the configuration's fixed dt, and the CFL dt
    of step() (3dmhdsub.h:36-106) computed every step, reduced over all
    threads (plane-parallel, the same DT as the serial order)."""
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle
    threads = threads or os.cpu_count() or 1
    sc = cpu_sample_case(case)
    st = initial_state(sc)
    o = oracle.OracleSim(sc, st, nthreads=threads)
    o.p.cfl_parallel = 1
    o.communicate()
    t1 = _time_oracle_steps(o, 1, None)
    n = max(1, min(50, int(target_s / max(t1, 1e-3))))
    secs = _time_oracle_steps(o, n, None)
    # the reference's default run mode: a CFL dt for every step
    o2 = oracle.OracleSim(sc, st, nthreads=threads)
    o2.p.cfl_parallel = 1
    o2.communicate()
    _time_oracle_steps(o2, 1, -1.0)
    ncfl = max(1, n // 2)
    secs_cfl = _time_oracle_steps(o2, ncfl, -1.0)
    return {"value": sc.cells * n / secs, "unit": METRIC, "cores": threads, "kind": "port",
            "flags": ORACLE_FLAGS,
            "sample": f"{sc.nPx}x{sc.nPy}x{sc.nPz} slab of the workload (same physics), {n} fixed-dt RK3 steps after "
                      f"1 warm-up, oracle/mhd_oracle.c with OpenMP over {threads} threads, {secs:.1f} s",
            "cfl_dt": {"value": sc.cells * ncfl / secs_cfl, "unit": METRIC, "steps": ncfl,
                       "ms_per_step": 1e3 * secs_cfl / ncfl, "cost_vs_fixed_dt": (secs_cfl / ncfl) / (secs / n) - 1.0,
                       "sample": f"the same slab, {ncfl} RK3 steps each with the CFL dt of step() "
                                 f"(3dmhdsub.h:36-106), the reduction over {threads} threads"}}


def run_reference(args, dist: Dist) -> None:
    if dist.rank != 0:
        return
    case = case_for(args.config)
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle
    threads = os.cpu_count() or 1
    sc = cpu_sample_case(case)
    st = initial_state(sc)
    o = oracle.OracleSim(sc, st, nthreads=threads)
    o.p.cfl_parallel = 1
    o.communicate()
    o.steps(max(1, args.warmup))
    secs = _time_oracle_steps(o, args.steps, None)
    value = sc.cells * args.steps / secs
    # the reference's default run mode (CFL dt every step) on the same slab
    o2 = oracle.OracleSim(sc, st, nthreads=threads)
    o2.p.cfl_parallel = 1
    o2.communicate()
    o2.steps(1, -1.0)
    secs_cfl = _time_oracle_steps(o2, args.steps, -1.0)
    sample = (f"each step: one RK3 step of a {sc.nPx}x{sc.nPy}x{sc.nPz} slab of the {case.name} workload "
              f"(same physics), oracle/mhd_oracle.c (bit-exact restatement of the reference) on {threads} threads")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(case, args),
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port", "sample": sample,
                             "flags": ORACLE_FLAGS,
                             "cfl_dt": {"value": sc.cells * args.steps / secs_cfl, "unit": METRIC,
                                        "ms_per_step": 1e3 * secs_cfl / args.steps,
                                        "sample": "the same slab and steps, each with the CFL dt of step() "
                                                  "(3dmhdsub.h:36-106)"}},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def workload_config(case, args) -> dict:
    return {"workload": f"{case.name}: plain method FP64, {case.nPx}x{case.nPy}x{case.nPz}, "
                        f"lMag={case.lMag} lRot={case.lRot} lShr={case.lShr}, fixed dt={case.dt}",
            "grid": [case.nPx, case.nPy, case.nPz], "cells": case.cells, "precision": "fp64",
            "path": "fused", "parallelism": f"replicas x{args.gpus}",
            "l2": "no flush: state of 24 fields x 545 MB is far larger than the 129 MB L2"}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args, dist: Dist) -> None:
    from mhd_gb300.sim import Simulation
    L = abi.load()
    abi.check(L.mhd_set_device(dist.local))
    case = case_for(args.config)
    st = initial_state(case)
    sim = Simulation(case, path="fused")
    sim.upload_state(st)
    sim.communicate()
    for _ in range(args.warmup):
        sim.step(case.dt)
    sim.sync()

    clocks = ClockSampler(dist.local)
    dist.barrier()
    sim.sync()
    clocks.start()
    sim.profile(True)
    sim.timer_start()
    for _ in range(args.steps):
        sim.step(case.dt)
    ms = sim.timer_stop()
    sub_ms, launches = sim.profile_read()
    sim.profile(False)
    clk = clocks.stop()
    dist.barrier()
    ms_max = dist.max(ms)
    value = dist.world * case.cells * args.steps / (ms_max / 1e3)

    # the reference's run mode: a CFL dt for every step, reduced on the device
    # into the record the substage kernels read (mhd_steps_cfl)
    sim.steps_cfl(1)
    sim.timer_start()
    _, dcfl = sim.steps_cfl(args.steps)
    ms_cfl = dist.max(sim.timer_stop())
    cfl_mode = {"value": dist.world * case.cells * args.steps / (ms_cfl / 1e3), "ms_per_step": ms_cfl / args.steps,
                "cost_vs_fixed_dt": ms_cfl / ms_max - 1.0, "last_dt": dcfl["dt"],
                "path": "mhd_steps_cfl: CFL reduction + 3 fused substages + BCON per step, one host sync per call"}

    # roofline of the fused substage kernel
    bytes_cell_step = algorithmic_bytes_per_cell_step(case)
    per_launch_bytes = case.cells * bytes_cell_step / 3.0
    avg_launch_s = (sub_ms / 1e3) / max(launches, 1)
    achieved_gbs = per_launch_bytes / avg_launch_s / 1e9
    peaks = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm_peak else "fallback"
    hbm_peak = hbm_peak or 6800.0
    fp64_peak = C.c_double(0.0)
    abi.check(L.mhd_fp64_peak(C.byref(fp64_peak)))
    key = (case.lMag, case.lRot, case.lShr)
    inst_cell = FP64_INST_PER_CELL_SUBSTAGE.get(key)
    tr = TRAFFIC_OVER_ALGORITHMIC.get(key)
    traffic = per_launch_bytes * tr if tr else None

    # end to end through the C ABI with pinned host buffers
    nf = case.nfields
    ncell = int(np.prod(case.shape))
    nbytes = nf * ncell * 8
    hp = C.c_void_p()
    abi.check(L.mhd_host_alloc(nbytes, C.byref(hp)))
    host = np.ctypeslib.as_array(C.cast(hp, C.POINTER(C.c_double)), shape=(nf * ncell,))
    for j, k in enumerate(STATE_FIELDS[:nf]):
        host[j * ncell:(j + 1) * ncell] = st[k].ravel()
    ptr = C.cast(hp, C.POINTER(C.c_double))
    e2e_steps = 0 if args.no_e2e else max(1, min(args.steps, args.e2e_steps))
    e2e_s = float("nan")
    percall_s = float("nan")
    serial_s = float("nan")
    if e2e_steps:
        # the steps of a host-resident driver: every step uploads its state
        # from pinned host memory and downloads the new state into it, the
        # transfers overlapped slab by slab and the steps enqueued back to back
        abi.check(L.mhd_steps_host(sim.ctx, 1, ptr, ptr, case.dt))
        dist.barrier()
        t = time.perf_counter()
        abi.check(L.mhd_steps_host(sim.ctx, e2e_steps, ptr, ptr, case.dt))
        e2e_s = dist.max(time.perf_counter() - t)
        # one blocking call per step
        dist.barrier()
        t = time.perf_counter()
        for _ in range(e2e_steps):
            abi.check(L.mhd_step_host(sim.ctx, ptr, ptr, case.dt))
        percall_s = dist.max(time.perf_counter() - t)
        # the same transfers one after another around mhd_step, for comparison
        dist.barrier()
        t = time.perf_counter()
        abi.check(L.mhd_upload_state(sim.ctx, ptr))
        sim.step(case.dt)
        abi.check(L.mhd_download_state(sim.ctx, ptr))
        serial_s = dist.max(time.perf_counter() - t)
    e2e_value = dist.world * case.cells * e2e_steps / e2e_s if e2e_steps else None
    L.mhd_host_free(hp)
    sim.close()

    # the batching (config 2) and precision (config 3) forms, measured in the
    # same run at their configured sizes and step counts
    forms = {}
    if dist.world == 1 and not args.no_forms:
        forms["batch"] = measure_batch(args.batch_steps, args.serial_steps)
        forms["precision"] = measure_precision(args.precision_steps)
        # the batch's FP64 rate per cell against one instance of the same physics
        # (lMag, 256x256x128 FP64 in the precision form)
        forms["batch"]["vs_single_instance_same_physics"] = forms["batch"]["value"] / forms["precision"]["fp64"]["value"]

    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(case)

    if dist.rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded polytrope + Gaussian T noise)",
        "config": workload_config(case, args),
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": e2e_steps, "ms_per_step": 1e3 * e2e_s / e2e_steps if e2e_steps else None,
                "path": "mhd_steps_host: pinned host state in and out every step, upload / 3 substages / "
                        "download overlapped over z slabs (uploads, one stream per substage, downloads), "
                        "the steps enqueued back to back",
                "per_call": {"value": dist.world * case.cells * e2e_steps / percall_s if e2e_steps else None,
                             "ms_per_step": 1e3 * percall_s / e2e_steps if e2e_steps else None,
                             "path": "mhd_step_host, one blocking call per step"},
                "serial_transfers": {"value": dist.world * case.cells / serial_s if e2e_steps else None,
                                     "ms_per_step": 1e3 * serial_s if e2e_steps else None,
                                     "path": "mhd_upload_state + mhd_step + mhd_download_state"}},
        "gpu_launches": 6 * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved_gbs / hbm_peak, "traffic": traffic,
                     "traffic_note": "ncu dram read+write of one launch at 256x256x128, scaled per cell",
                     "kernel": "k_substage (fused RK3 substage)", "peak_source": f"{peak_src} hbm_gbs",
                     "algorithmic_bytes_per_cell_step": bytes_cell_step,
                     "avg_launch_ms": 1e3 * avg_launch_s, "launches": launches},
        "fp64": {"bound": "fp64 pipe", "unit": "G FP64 inst/s",
                 "achieved": inst_cell * case.cells / avg_launch_s / 1e9 if inst_cell else None,
                 "peak": fp64_peak.value * 1e3 / 2.0,
                 "frac": (inst_cell * case.cells / avg_launch_s / 1e9) / (fp64_peak.value * 1e3 / 2.0)
                         if inst_cell and fp64_peak.value > 0 else None,
                 "inst_per_cell_substage": inst_cell, "peak_tflops_measured": fp64_peak.value,
                 "note": "the FP64 pipe (measured DFMA roof), not HBM, bounds the fused FP64 kernel on GB300"},
        "clocks": clk,
        "adaptive_cfl": cfl_mode,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    line.update(forms)
    print(json.dumps(line), flush=True)


# FP64-pipe instructions per interior cell per substage of the fused kernel,
# keyed by (lMag, lRot, lShr): ncu's sm__inst_executed_pipe_fp64 share x the
# 2/clk/SM pipe rate x elapsed cycles / cells, from the 256x256x128 capture in
# profiles/k_substage_fp64_config1physics_256x256x128.md.
FP64_INST_PER_CELL_SUBSTAGE: dict = {(True, True, True): 200.5}
# DRAM traffic over algorithmic bytes of one k_substage launch, measured by ncu
# at 256x256x128 (2.274 GB / 2.282 GB); applied to the full-size average launch.
TRAFFIC_OVER_ALGORITHMIC = {(True, True, True): 2.274 / 2.282}


# ---------------------------------------------------------------------------
# precision form: FP32 storage vs the FP64 path on the 256x256x128 case
# ---------------------------------------------------------------------------
def run_precision(args, dist: Dist) -> None:
    L = abi.load()
    abi.check(L.mhd_set_device(dist.local))
    out = measure_precision(args.precision_steps)
    if dist.rank == 0:
        print(json.dumps(out), flush=True)


def measure_precision(nsteps: int) -> dict:
    """Config 3: 256x256x128 lMag, noise 1e-2, `nsteps` fixed-dt steps with
    FP64 storage and with FP32 storage (FP64 RK register, EOS and
    reductions); per-field errors of the FP32 state against the FP64 one,
    mass / energy drift and max |div B| before and after."""
    from mhd_gb300.sim import Simulation
    case = config3()
    st = initial_state(case)
    res = {}
    for prec in ("fp64", "fp32"):
        sim = Simulation(case, precision=prec)
        sim.upload_state(st)
        sim.communicate()
        d0 = sim.diagnostics()
        for _ in range(3):
            sim.step(case.dt)
        sim.upload_state(st)
        sim.communicate()
        sim.set_time(0.0, 0)
        sim.sync()
        sim.profile(True)
        sim.timer_start()
        sim.steps(nsteps, case.dt)
        ms = sim.timer_stop()
        sub_ms, launches = sim.profile_read()
        sim.profile(False)
        d1 = sim.diagnostics(check=False)
        state = sim.download_state()
        # the reference's run mode on the same context: 100 steps with a CFL dt each,
        # reduced on the device into the record the substages read
        sim.timer_start()
        sim.steps_cfl(100)
        ms_cfl = sim.timer_stop()
        res[prec] = {"state": state, "ms": ms, "sub_ms": sub_ms, "launches": launches,
                     "d0": d0, "d1": d1, "ms_cfl": ms_cfl}
        sim.close()
    errs = {}
    for k in STATE_FIELDS:
        a = res["fp32"]["state"][k][1:-1, 1:-1, 1:-1]
        b = res["fp64"]["state"][k][1:-1, 1:-1, 1:-1]
        nb = np.linalg.norm(b)
        errs[k] = {"l2_rel": float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b)),
                   "linf_rel": float(np.abs(a - b).max() / np.abs(b).max()) if np.abs(b).max() > 0 else None}
    out = {"form": "precision", "metric": METRIC, "unit": METRIC, "steps": nsteps,
           "config": {"workload": f"{case.name}: lMag, noise 1e-2, dt {case.dt}, {nsteps} steps"}}
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs") or 6800.0
    for prec in ("fp64", "fp32"):
        r = res[prec]
        bytes_cs = 640.0 if prec == "fp64" else 448.0
        avg = r["sub_ms"] / 1e3 / max(r["launches"], 1)
        out[prec] = {"value": case.cells * nsteps / (r["ms"] / 1e3), "ms_per_step": r["ms"] / nsteps,
                     "algorithmic_bytes_per_cell_step": bytes_cs,
                     "substage_gbs": case.cells * bytes_cs / 3 / avg / 1e9,
                     "substage_hbm_frac": case.cells * bytes_cs / 3 / avg / 1e9 / hbm,
                     "drift": {k: r["d1"][k] / r["d0"][k] - 1.0 if r["d0"][k] else None
                               for k in ("total_mass", "total_energy")},
                     "max_divb": [r["d0"]["max_divb"], r["d1"]["max_divb"]],
                     "adaptive_cfl": {"value": case.cells * 100 / (r["ms_cfl"] / 1e3),
                                      "ms_per_step": r["ms_cfl"] / 100,
                                      "cost_vs_fixed_dt": (r["ms_cfl"] / 100) / (r["ms"] / nsteps) - 1.0}}
    out["speedup_fp32_over_fp64"] = out["fp32"]["value"] / out["fp64"]["value"]
    out["fp32"]["vs_plain_fp64"] = out["speedup_fp32_over_fp64"]
    out["fp64"]["vs_plain_fp64"] = 1.0
    out["errors_fp32_vs_fp64"] = errs
    out["max_l2_rel"] = max(e["l2_rel"] for e in errs.values())
    out["value"] = out["fp32"]["value"]
    out["ms_per_step"] = out["fp32"]["ms_per_step"]
    out["vs_plain_fp64"] = out["speedup_fp32_over_fp64"]
    return out


# ---------------------------------------------------------------------------
# batching form: 64 uneven instances, persistent launch per substage, graphs
# ---------------------------------------------------------------------------
def run_batch(args, dist: Dist) -> None:
    L = abi.load()
    abi.check(L.mhd_set_device(dist.local))
    out = measure_batch(args.batch_steps, args.serial_steps)
    if dist.rank == 0:
        print(json.dumps(out), flush=True)


def measure_batch(nsteps: int, serial_steps: int) -> dict:
    """Config 2: 64 instances with the configuration's draw of sizes, seeds,
    1/Re and Bz0, `nsteps` batched steps (one persistent launch per substage,
    graph-captured, autotuned tile) with FP64 and with FP32 storage, against
    the same instances stepped one after another on the plain FP64 path (a
    bounded sample of `serial_steps` steps, scaled to `nsteps`)."""
    from mhd_gb300.sim import Batch, Simulation
    cases = config2_batch()
    sims = []
    for c in cases:
        s = Simulation(c)
        s.upload_state(initial_state(c))
        s.communicate()
        sims.append(s)
    cells = sum(c.cells for c in cases)
    b = Batch(sims)
    chosen, tile_ms = b.autotune()
    zrange = b.zrange()
    b.steps(3)
    b.sync()
    sims[0].timer_start()
    t = time.perf_counter()
    b.steps(nsteps)
    b.sync()
    secs = time.perf_counter() - t
    b.close()
    # the plain single-instance path, instance after instance (a bounded sample of steps)
    serial_steps = max(1, min(nsteps, serial_steps))
    for s in sims:
        s.steps(2, s.case.dt)
        s.sync()
    t = time.perf_counter()
    for s in sims:
        s.steps(serial_steps, s.case.dt)
        s.sync()
    serial_secs = (time.perf_counter() - t) * nsteps / serial_steps
    for s in sims:
        s.close()
    # the same instances with FP32 storage, batched
    sims32 = []
    for c in cases:
        s = Simulation(c, precision="fp32")
        s.upload_state(initial_state(c))
        s.communicate()
        sims32.append(s)
    b32 = Batch(sims32)
    _, tile32_ms = b32.autotune()
    zrange32 = b32.zrange()
    b32.steps(3)
    b32.sync()
    t = time.perf_counter()
    b32.steps(nsteps)
    b32.sync()
    secs32 = time.perf_counter() - t
    b32.close()
    for s in sims32:
        s.close()
    out = {"form": "batch", "metric": METRIC, "unit": METRIC, "instances": len(cases), "steps": nsteps,
           "fp32_storage_batched": {"value": cells * nsteps / secs32, "ms_per_step": 1e3 * secs32 / nsteps,
                                    "vs_plain_fp64_serial": serial_secs / secs32,
                                    "vs_fp64_batched": secs / secs32},
           "cells_per_step": cells, "dtype": "f64",
           "value": cells * nsteps / secs, "ms_per_step": 1e3 * secs / nsteps,
           "autotune": {"chosen": ["32x4", "32x8", "16x8"][chosen], "zrange": zrange,
                        "ms_per_step_by_tile": tile_ms, "fp32_zrange": zrange32,
                        "fp32_ms_per_step": tile32_ms[0]},
           "plain_serial": {"value": cells * nsteps / serial_secs, "ms_per_step": 1e3 * serial_secs / nsteps,
                            "sample_steps": serial_steps},
           "speedup_vs_plain_serial": serial_secs / secs,
           "config": {"workload": "64 FP64 MHD instances, nx=ny in {32,48,64,96,128}, nz in {32,64}, "
                                  "1/Re log-uniform [3e-3,3e-2], Bz0 log-uniform [1e-4,1e-2]"}}
    out["vs_plain_fp64"] = out["speedup_vs_plain_serial"]
    out["fp32_storage_batched"]["vs_plain_fp64"] = out["fp32_storage_batched"]["vs_plain_fp64_serial"]
    return out


# ---------------------------------------------------------------------------
# serving form: Poisson request stream, continuous batching under an HBM budget
# ---------------------------------------------------------------------------
def run_serve(args, dist: Dist) -> None:
    """Config 4: the Poisson request stream served with continuous batching
    under a 150 GB HBM budget.  Baseline: the same requests one after another
    on the plain FP64 path -- all of them for a short stream, else a seeded
    random sample of --serve-serial-sample requests, timed per cell-step and
    scaled to the stream's cell-steps."""
    from mhd_gb300.serve import Server, poisson_requests, run_serial
    L = abi.load()
    abi.check(L.mhd_set_device(dist.local))
    n = args.serve_requests
    smin, smax = max(1, 50 // args.serve_step_scale), max(2, 2000 // args.serve_step_scale)

    def stream():
        return poisson_requests(n, rate=20.0, seed=4, steps=(smin, smax), fp32_fraction=0.5)

    log = open(args.serve_progress, "a") if args.serve_progress else None

    def progress(d):
        if log:
            log.write(json.dumps(d) + "\n")
            log.flush()
    reqs = stream()
    srv = Server(150 << 30, quantum=25, policy="srpt", progress=progress)
    st = srv.run(reqs, realtime=True)
    progress({"done": "srpt", **{k: st[k] for k in ("value", "wall_s", "tts_p50_s", "tts_p99_s")}})
    fifo = None
    if args.serve_fifo:
        fifo = Server(150 << 30, quantum=25, policy="fifo", tile=st["tile"]).run(stream(), realtime=True)
    # baseline: the same requests one after another on the plain FP64 path
    all_reqs = stream()
    total_cs = sum(r.case.cells * r.steps for r in all_reqs)
    if args.serve_serial_sample and args.serve_serial_sample < n:
        rng = np.random.default_rng(7)
        pick = sorted(rng.choice(n, size=args.serve_serial_sample, replace=False))
        sample = [all_reqs[i] for i in pick]
        base = run_serial(sample)
        base = {"value": base["value"], "sample_requests": len(sample), "sample_wall_s": base["wall_s"],
                "sample_cell_steps": base["cell_steps"], "wall_s_scaled": total_cs / base["value"],
                "note": "seeded random sample of the stream, timed per cell-step, scaled to the whole stream"}
    else:
        base = run_serial(all_reqs)
    steps_ms = [r.steps for r in reqs]
    out = {"form": "serve", "metric": METRIC, "unit": METRIC, "requests": n, "rate_per_s": 20.0,
           "steps_range": [smin, smax], "hbm_budget_gb": 150, "cell_steps": total_cs,
           "value": st["value"], "wall_s": st["wall_s"], "tts_p50_s": st["tts_p50_s"],
           "tts_p99_s": st["tts_p99_s"], "max_resident": st["max_resident"], "tile": st["tile"],
           "zrange": st["zrange"], "batch_rebuilds": st["batch_rebuilds"], "policy": st["policy"],
           "target_cells": srv.target_cells, "mean_steps": float(np.mean(steps_ms)),
           "serial_plain_fp64": base, "throughput_vs_serial": st["value"] / base["value"],
           "config": {"workload": f"Poisson stream of {n} simulations at 20/s, grids log-uniform 32^3..256^2x128, "
                                  f"steps uniform [{smin},{smax}]"
                                  + (f" (the configured [50,2000] / {args.serve_step_scale})"
                                     if args.serve_step_scale != 1 else "")
                                  + ", half FP32 storage, random seeds and 1/Re"}}
    if fifo:
        out["fifo"] = {k: fifo[k] for k in ("value", "wall_s", "tts_p50_s", "tts_p99_s", "max_resident",
                                            "batch_rebuilds")}
    if dist.rank == 0:
        print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=["config1", "config0", "mid"], default="config1")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--form", choices=["plain", "precision", "batch", "serve"], default="plain")
    ap.add_argument("--batch-steps", type=int, default=500)
    ap.add_argument("--serial-steps", type=int, default=20)
    ap.add_argument("--serve-requests", type=int, default=200)
    ap.add_argument("--serve-step-scale", type=int, default=10)
    ap.add_argument("--serve-serial-sample", type=int, default=0,
                    help="time the serial baseline on this many sampled requests (0 = all)")
    ap.add_argument("--serve-fifo", action="store_true", help="also serve the stream first come, first served")
    ap.add_argument("--serve-progress", default=None, help="append running totals (JSON lines) to this file")
    ap.add_argument("--precision-steps", type=int, default=1000)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the batch and precision keys of the default line")
    args = ap.parse_args()
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        elif args.form == "precision":
            run_precision(args, dist)
        elif args.form == "batch":
            run_batch(args, dist)
        elif args.form == "serve":
            run_serve(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
