"""Continuous-batching server for independent 3dmhd simulations on one GPU.

Requests (a grid, a step count, a precision, a seed) arrive over time.  The
server admits a waiting request as soon as its device memory fits in the HBM
budget next to the simulations already resident, uploads its initial state,
and steps every resident simulation together: simulations with the same
precision and switch set form one ragged batch (one persistent launch per RK3
substage over all of their tiles, each step a CUDA graph); the FP64 and the
FP32-storage batches run on their own streams, so their kernels overlap.  A simulation
leaves when its step count is reached; its memory is freed at once and the
next waiting request takes the slot.  Each step of each simulation computes
exactly what it would compute alone (the per-cell arithmetic does not depend
on the mix), so results are the same alone and in the mix.

Admission policy: "fifo" admits in arrival order whenever memory fits, so
every admitted simulation shares the GPU with all others until the end;
"srpt" (shortest remaining processing time first) admits the waiting
requests with the least work (cells x steps) first and keeps only as many
resident as needed to fill the GPU (target_cells of resident work), which
cuts the typical time-to-solution without lowering the throughput.

Time-to-solution of a request = completion time - arrival time; the server
reports p50 / p99 of it and the aggregate cell-RK3-updates/s.
"""
from __future__ import annotations

import dataclasses
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from .case import Case, STATE_FIELDS, initial_state
from .sim import Batch, Simulation

DEFAULT_TILE = 2  # the 16x8 batch tile, the shape of the single-instance kernel


@dataclass
class Request:
    rid: int
    case: Case
    steps: int
    precision: str = "fp64"   # "fp64" or "fp32"
    arrival: float = 0.0      # seconds after the start of the run
    t_admit: float | None = None
    t_done: float | None = None
    result: dict | None = None


def device_bytes_estimate(case: Case, precision: str) -> int:
    """Device memory a simulation needs on the fused path."""
    n = case.nx * case.ny * case.nz
    if precision == "fp64":
        fields = 24 + (8 if case.lShr else 0)  # U[2], Z, and the right-hand-side block for FT
        return n * 8 * fields + 64 * 1024
    return n * (4 * 16 + 8 * 8 + (8 if case.lShr else 0)) + 64 * 1024


def poisson_requests(n: int, rate: float, seed: int = 0, grid_min=(32, 32, 32), grid_max=(256, 256, 128),
                     steps=(50, 2000), fp32_fraction: float = 0.5, re_range=(3e-3, 3e-2),
                     base: Case | None = None) -> list:
    """Request stream: Poisson arrivals at `rate` per second, grids
    log-uniform between grid_min and grid_max (nx = ny), step counts uniform,
    mixed precision, random seeds and 1/Re log-uniform."""
    rng = np.random.default_rng(seed)
    base = base or Case(nPx=32, nPy=32, nPz=32, lMag=True)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        lx = np.exp(rng.uniform(np.log(grid_min[0]), np.log(grid_max[0])))
        lz = np.exp(rng.uniform(np.log(grid_min[2]), np.log(grid_max[2])))
        nxy = int(max(grid_min[0], min(grid_max[0], round(lx / 8) * 8)))
        nz = int(max(grid_min[2], min(grid_max[2], round(lz / 4) * 4)))
        ore = np.exp(rng.uniform(np.log(re_range[0]), np.log(re_range[1])))
        case = base.replace(nPx=nxy, nPy=nxy, nPz=nz, seed=int(rng.integers(1 << 30)), RE=float(1.0 / ore),
                            name=f"req{i}")
        nsteps = int(rng.integers(steps[0], steps[1] + 1))
        prec = "fp32" if rng.random() < fp32_fraction else "fp64"
        out.append(Request(rid=i, case=case, steps=nsteps, precision=prec, arrival=t))
    return out


def init_state(sim, case: Case, precision: str, device_init: bool) -> None:
    """Initial state of a request: generated on the GPU (both precisions), or
    numpy's on the host and uploaded."""
    if device_init:
        sim.init_on_device()
    else:
        sim.upload_state(initial_state(case))
    sim.communicate()


class _Resident:
    def __init__(self, req: Request, sim: Simulation, nbytes: int):
        self.req = req
        self.sim = sim
        self.remaining = req.steps
        self.nbytes = nbytes


class Server:
    """Admits requests under an HBM budget and steps the resident ones together.

    quantum: at most this many steps are queued per resident simulation
    between scheduling decisions (admissions and completions happen between
    quanta); a simulation with fewer steps left takes only those and drops
    out of the batch's work for the rest of the quantum, so one nearly
    finished request does not shorten the quantum of all others.  tile: FP64
    batch tile shape (None = the 16x8 tile until an FP64 batch holds at least
    a quarter of target_cells, then the autotuner's choice of tile shape and
    z range on that batch, kept for the rest of the run: a tuning on the
    first, often tiny, batch would fix a shape that suits a handful of small
    grids); FP32-storage batches tune their z range the same way.  The
    autotuner's scratch copy of the batch counts against the HBM budget while
    it runs: when it does not fit, the batch keeps the default and tuning is
    tried again at the next rebuild.  progress: optional callable receiving a
    dict of running totals every progress_s seconds."""

    def __init__(self, hbm_budget_bytes: int, quantum: int = 25, tile: int | None = None,
                 keep_results: bool = False, device_init: bool = True, policy: str = "srpt",
                 target_cells: int = 64_000_000, progress=None, progress_s: float = 30.0,
                 balance: bool = True, rates: dict | None = None):
        if policy not in ("fifo", "srpt"):
            raise ValueError(f"unknown admission policy {policy!r}")
        self.policy = policy
        self.target_cells = int(target_cells)
        self.resident_cells = 0
        self.budget = int(hbm_budget_bytes)
        self.quantum = int(quantum)
        self.tile = tile
        self.tuned = {"fp64": tile is not None, "fp32": False}
        self.zrange = {"fp64": None, "fp32": None}
        self.balance = balance
        # nominal cell-RK3-updates/s of a batch per precision (the 64-instance batch, measured:
        # 7.97e8 and 4.29e9)
        self.rates = dict(rates or {"fp64": 8.0e8, "fp32": 4.3e9})
        self.progress = progress
        self.progress_s = float(progress_s)
        self.completed = 0
        self.tune_skipped = 0
        self.keep_results = keep_results
        self.device_init = device_init
        self.used = 0
        self.resident: dict[int, _Resident] = {}
        self.batches: dict = {}
        self.batch_members: dict = {}
        self.cell_steps = 0
        self.admissions = 0
        self.max_resident = 0
        self.batch_rebuilds = 0

    # -- membership ------------------------------------------------------
    def _admit(self, req: Request, now: float) -> bool:
        need = device_bytes_estimate(req.case, req.precision)
        if self.used + need > self.budget:
            return False
        if self.policy == "srpt" and self.resident and self.resident_cells >= self.target_cells:
            return False
        sim = Simulation(req.case, precision=req.precision)
        init_state(sim, req.case, req.precision, self.device_init)
        self.used += need
        self.resident_cells += req.case.cells
        req.t_admit = now
        self.resident[req.rid] = _Resident(req, sim, need)
        self.admissions += 1
        self.max_resident = max(self.max_resident, len(self.resident))
        return True

    def _finish(self, r: _Resident, now: float) -> None:
        if self.keep_results:
            r.req.result = r.sim.download_state()
        else:
            r.sim.sync()
        r.sim.close()
        self.used -= r.nbytes
        self.resident_cells -= r.req.case.cells
        r.req.t_done = now
        self.completed += 1
        del self.resident[r.req.rid]

    def _groups(self):
        g = {}
        for rid, r in self.resident.items():
            key = (r.req.precision, r.req.case.lMag, r.req.case.lRot, r.req.case.lShr)
            g.setdefault(key, []).append(rid)
        return g

    def _sync_batches(self) -> None:
        groups = self._groups()
        for key in list(self.batches):
            if key not in groups or self.batch_members[key] != groups[key]:
                self.batches[key].close()
                del self.batches[key]
                del self.batch_members[key]
        for key, rids in groups.items():
            if key not in self.batches:
                b = Batch([self.resident[r].sim for r in rids])
                prec = key[0]
                if not self.tuned[prec] and sum(self.resident[r].sim.case.cells for r in rids) >= self.target_cells // 4:
                    if self.used + b.autotune_bytes() <= self.budget:
                        tile, _ = b.autotune(report=False)
                        if prec == "fp64":
                            self.tile = tile
                        self.zrange[prec] = b.zrange()
                        self.tuned[prec] = True
                    else:
                        self.tune_skipped += 1
                if prec == "fp64":
                    b.set_tile(self.tile if self.tile is not None else DEFAULT_TILE)
                else:
                    b.set_tile(0)
                if self.zrange[prec] is not None:
                    b.set_zrange(self.zrange[prec])
                self.batches[key] = b
                self.batch_members[key] = list(rids)
                self.batch_rebuilds += 1

    # -- one scheduling quantum --------------------------------------------
    def _quanta(self) -> dict:
        """Steps per batch for the next quantum.  The batch with the longest
        estimated step (cells / nominal rate of its precision) takes `quantum`
        steps; with balance on, every other batch takes as many steps as fit
        in the same time (at most 8 x quantum), so the FP32-storage batch,
        about five times faster per cell, does not idle while the FP64 batch
        finishes its quantum."""
        est = {key: sum(self.resident[rid].req.case.cells for rid in rids) / self.rates[key[0]]
               for key, rids in self.batch_members.items()}
        longest = max(est.values())
        out = {}
        for key, rids in self.batch_members.items():
            q = self.quantum
            if self.balance and est[key] > 0:
                q = int(min(8 * self.quantum, max(self.quantum, round(self.quantum * longest / est[key]))))
            out[key] = min(q, max(self.resident[rid].remaining for rid in rids))
        return out

    def _launch(self) -> tuple[dict, dict]:
        """Queue each batch's quantum, every simulation taking at most its
        remaining steps (no wait); returns the steps per batch and the
        requests of each batch."""
        if not self.batch_members:
            return {}, {}
        qs = self._quanta()
        members = {key: list(rids) for key, rids in self.batch_members.items()}
        for key, b in self.batches.items():
            b.steps_limited(qs[key], [self.resident[rid].remaining for rid in members[key]])
        return qs, members

    def _complete(self, qs: dict, members: dict) -> int:
        """Wait for the queued quantum and account its steps; returns the steps
        taken by the batch whose quantum was estimated to take longest (the
        virtual clock's measure of the quantum)."""
        for b in self.batches.values():
            b.sync()
        longest, steps = -1.0, 0
        for key, rids in members.items():
            took_cells, took_max = 0, 0
            for rid in rids:
                r = self.resident[rid]
                took = min(qs[key], r.remaining)
                r.remaining -= took
                self.cell_steps += r.req.case.cells * took
                took_cells += r.req.case.cells * took
                took_max = max(took_max, took)
            t = took_cells / self.rates[key[0]]
            if t > longest:
                longest, steps = t, took_max
        return steps

    def run(self, requests: list, realtime: bool = True, virtual_step_s: float = 1e-3) -> dict:
        """Serve `requests`.  realtime=False replaces the wall clock by a
        virtual one that advances virtual_step_s per queued step, so a run's
        admissions are reproducible.

        Each round queues one quantum for the batched simulations, then
        admits waiting requests while the GPU works on it (creating a context
        and its initial state is host work), waits, retires the finished
        simulations and rebuilds the batches whose membership changed."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        future = deque(reqs)
        waiting: deque = deque()
        t0 = time.perf_counter()
        clock = (lambda: time.perf_counter() - t0) if realtime else None
        virtual = 0.0
        next_report = self.progress_s
        while future or waiting or self.resident:
            now = clock() if realtime else virtual
            if self.progress and now >= next_report:
                next_report = now + self.progress_s
                self.progress({"t_s": now, "completed": self.completed, "resident": len(self.resident),
                               "waiting": len(waiting), "future": len(future), "cell_steps": self.cell_steps,
                               "value": self.cell_steps / now if now > 0 else None,
                               "batch_rebuilds": self.batch_rebuilds})
            while future and future[0].arrival <= now:
                waiting.append(future.popleft())
            if self.policy == "srpt" and len(waiting) > 1:
                waiting = deque(sorted(waiting, key=lambda r: (r.case.cells * r.steps, r.arrival)))
            qs, members = self._launch()
            changed = False
            while waiting and self._admit(waiting[0], now):
                waiting.popleft()
                changed = True
            if not self.resident:
                if waiting and not future:
                    raise RuntimeError(f"request {waiting[0].rid} does not fit the HBM budget on its own")
                if future:
                    nxt = future[0].arrival
                    if realtime:
                        time.sleep(max(0.0, nxt - clock()))
                    else:
                        virtual = nxt
                continue
            if members:
                took = self._complete(qs, members)
                if not realtime:
                    virtual += took * virtual_step_s
            now = clock() if realtime else virtual
            done = [r for r in self.resident.values() if r.remaining <= 0]
            for r in done:
                self._finish(r, now)
            if changed or done:
                self._sync_batches()
        wall = (clock() if realtime else virtual)
        for b in self.batches.values():
            b.close()
        self.batches.clear()
        tts = np.array([r.t_done - r.arrival for r in reqs])
        return {"requests": len(reqs), "policy": self.policy, "wall_s": wall, "cell_steps": self.cell_steps,
                "value": self.cell_steps / wall if wall > 0 else None,
                "tts_p50_s": float(np.percentile(tts, 50)), "tts_p99_s": float(np.percentile(tts, 99)),
                "max_resident": self.max_resident, "batch_rebuilds": self.batch_rebuilds,
                "tile": self.tile if self.tile is not None else DEFAULT_TILE, "zrange": dict(self.zrange),
                "tune_skipped": self.tune_skipped}


def run_serial(requests: list, device_init: bool = True) -> dict:
    """The same requests one after another on the plain single-instance FP64
    path (the baseline of the serving form)."""
    t0 = time.perf_counter()
    cs = 0
    for req in requests:
        sim = Simulation(req.case, precision="fp64")
        init_state(sim, req.case, "fp64", device_init)
        sim.steps(req.steps, req.case.dt)
        sim.sync()
        sim.close()
        cs += req.case.cells * req.steps
    wall = time.perf_counter() - t0
    return {"wall_s": wall, "cell_steps": cs, "value": cs / wall}
