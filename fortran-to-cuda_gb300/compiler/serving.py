"""Serving advection jobs with continuous batching.

A job asks for ``steps`` forward-Euler steps (dt = 0.1, with the boundary fill
after each) of an advection instance: seeded sine-mode U, V, W and 0-3
scalars on an nx x ny x nz grid. The server keeps every admitted job's fields
resident on the device (two buffer sets, ping-pong) until its last step. Each
tick advances the jobs with the least remaining work, up to about 4 M grid
points, by one step: per scalar count one persistent batched launch over the
union of their tiles (``f2c_batch_*``) and one batched boundary fill. Jobs are
admitted as they arrive while slots and memory allow (a device-memory budget,
150 GB by default); their fields are generated on a side stream and they join
the ticks once ready, so their steps overlap on the device with the running
jobs' steps. Every job's arithmetic is the single-instance kernel's, so a job's
result is the same alone and in any mix, bit for bit.

The open-loop arrival stream and the job sizes follow the serving
configuration: Poisson arrivals at a given rate; nx and ny drawn independently
log-uniform in [48, 320], nz log-uniform in [24, 128]; 0-3 scalars and 1-100
steps uniform. ``SerialServer`` gives the comparison: the same stream served
one job at a time through the single-instance path, in wall-clock time with
the same per-job work; ``serial_timeline`` models it from device times alone.
"""

from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import native
from . import workloads as wl

DT = 0.1
BUDGET_BYTES = 150 * 10**9
MAX_ACTIVE = 256
# grid points advanced per tick before further jobs wait for the next tick: about 1 ms of work. Measured on
# GB300 (50 jobs per rate): ticks of 4M points keep throughput equal to serving one job at a time and halve the
# median latency at low rates; larger ticks trade median latency for a few percent of throughput, and 2M-point
# ticks leave the GPU waiting for the host
TICK_POINTS = 4_000_000
BURST = 8  # ticks issued at once while the selection holds


@dataclass
class Job:
    ident: int
    arrival: float              # seconds after the stream starts
    nx: int
    ny: int
    nz: int
    nscalar: int
    steps: int
    seed: int
    halo: int = 2
    # server state
    ready: object = None        # event: the fields generated at admission are complete
    admitted: float = -1.0
    finished: float = -1.0
    done: int = 0
    buffers: list = field(default_factory=list)   # [set A tensors, set B tensors]
    grid: object = None
    result: list = field(default_factory=list)

    @property
    def geometry(self) -> wl.Geometry:
        return wl.Geometry(self.nx, self.ny, self.nz, halo=self.halo)

    @property
    def points(self) -> int:
        return self.nx * self.ny * self.nz

    def device_bytes(self) -> int:
        g = self.geometry
        return 2 * (3 + self.nscalar) * int(np.prod(g.shape)) * 8


def tick_chunk_depth(shapes, sms: int) -> int:
    """One z-chunk depth for a tick's batch: deep chunks (up to 32 levels) while the tick has work for four
    CTAs per SM, shallower (down to 2) for small ticks, so that their tiles still spread over every SM."""
    columns = sum(((nx + 31) // 32) * ((ny + 7) // 8) * nz for (nx, ny, nz) in shapes)
    return int(min(32, max(2, -(-columns // (4 * sms)))))


def log_uniform_int(rng, lo, hi):
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def poisson_jobs(count: int, rate: float, seed: int = 0) -> list[Job]:
    """An open-loop stream: exponential inter-arrival gaps; per job draws in the order nx, ny, nz, scalars, steps."""
    rng = np.random.default_rng(seed)
    jobs, t = [], 0.0
    for n in range(count):
        t += float(rng.exponential(1.0 / rate))
        nx = log_uniform_int(rng, 48, 320)
        ny = log_uniform_int(rng, 48, 320)
        nz = log_uniform_int(rng, 24, 128)
        nscalar = int(rng.integers(0, 4))
        steps = int(rng.integers(1, 101))
        jobs.append(Job(n, t, nx, ny, nz, nscalar, steps, seed=10_000 + n))
    return jobs


class Server:
    """Continuous-batching server on one GPU (``torch`` provides device memory and the stream).

    A tick advances the selected jobs by one step: per scalar count, one
    batched step over all their tiles and one batched boundary fill. A plan
    depends only on which jobs step and which of their two buffer sets is
    current, so it repeats every other tick while the selection holds: plans
    are cached (each with its own device workspace, built once without
    stalling the stream through ``prepare_async``), ticks are ordered by
    events, and the host runs at most ``depth`` ticks ahead of the device. A
    job whose last step is issued is retired once that tick's event has
    completed.

    Which jobs step in a tick: those with the least remaining work (steps left
    x points) first, until the tick holds ``tick_points`` grid points; the rest
    stay resident and wait (shortest remaining work first, so short jobs leave
    early while every tick still fills the GPU). ``tick_points=None`` steps every
    active job every tick.
    """

    def __init__(self, torch, budget_bytes: int = BUDGET_BYTES, max_active: int = MAX_ACTIVE, keep_results=False,
                 depth: int = 4, tick_points: int | None = TICK_POINTS):
        self.torch = torch
        self.tick_points = tick_points
        self.budget = budget_bytes
        self.max_active = max_active
        self.keep_results = keep_results
        self.depth = depth
        self.stream = torch.cuda.Stream()
        self.admit_stream = torch.cuda.Stream()  # admissions run beside the ticks, not between them
        self.active: list[Job] = []
        self.claimed = 0
        self.ticks = 0
        self.launches = 0
        self.sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        self.plans = {}        # (scalars, ((job, parity), ...)) -> (Batch, workspace, staging), most recent last
        self.plan_builds = 0
        self.inflight = []     # (event, plans used, jobs finishing at this tick)

    # -- job lifetime ---------------------------------------------------------------------------
    def _admit(self, job: Job, now: float) -> None:
        torch = self.torch
        geo = job.geometry
        with torch.cuda.stream(self.admit_stream):
            first = wl.advection_fields_device(geo, job.seed, job.nscalar, torch)
            second = [torch.empty_like(t) for t in first]
        for t in first + second:
            t.record_stream(self.stream)
        job.grid = native.make_grid(geo.nx, geo.ny, geo.nz, geo.halo, geo.dx, geo.dy, geo.dz)
        kinds = [0, 0, 1] + [0] * job.nscalar
        native.halo_fill(job.grid, [t.data_ptr() for t in first], kinds, stream=self.admit_stream.cuda_stream)
        job.ready = torch.cuda.Event()
        job.ready.record(self.admit_stream)
        self.launches += 1
        job.buffers = [first, second]
        job.admitted = now
        self.claimed += job.device_bytes()
        self.active.append(job)

    def _retire(self, job: Job, now: float) -> None:
        current = job.buffers[job.done % 2]
        if self.keep_results:
            job.result = [t.cpu().numpy() for t in current]
        else:
            current[0].view(-1)[:1].cpu()  # the job's answer is read back (one value; fields stay for inspection)
        job.finished = now
        job.buffers = []
        self.claimed -= job.device_bytes()

    def fits(self, job: Job) -> bool:
        return len(self.active) < self.max_active and self.claimed + job.device_bytes() <= self.budget

    def _plan(self, nscalar: int, jobs: list[Job]):
        """The cached plan of one group's step (built on first use; the 16 most recent are kept)."""
        key = (nscalar, tuple((job.ident, job.done % 2) for job in jobs))
        plan = self.plans.pop(key, None)
        if plan is None:
            torch = self.torch
            grids, fields = [], []
            for job in jobs:
                src, dst = job.buffers[job.done % 2], job.buffers[1 - job.done % 2]
                p, q = [t.data_ptr() for t in src], [t.data_ptr() for t in dst]
                grids.append(job.grid)
                fields.append(native.make_fields(*p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:],
                                                 mode=native.ADVANCE, dt=DT))
            kz = tick_chunk_depth([(j.nx, j.ny, j.nz) for j in jobs], self.sms)
            batch = native.Batch(grids, fields, kz=[kz] * len(jobs))
            need = batch.workspace_bytes()
            workspace = torch.empty(need, dtype=torch.uint8, device="cuda")
            staging = torch.empty(need, dtype=torch.uint8, pin_memory=True)
            batch.prepare_async(workspace.data_ptr(), need, staging.data_ptr(), self.stream.cuda_stream)
            plan = (batch, workspace, staging)
            self.plan_builds += 1
        self.plans[key] = plan
        while len(self.plans) > 16:  # ticks still in flight hold their own references
            self.plans.pop(next(iter(self.plans)))
        return plan

    # -- one tick: every active job advances one step --------------------------------------------
    def _ready(self) -> list[Job]:
        """Active jobs whose admission has completed."""
        out = []
        for job in self.active:
            if job.ready is not None and job.ready.query():
                job.ready = None
            if job.ready is None:
                out.append(job)
        return out

    def select(self) -> list[Job]:
        """The jobs that step in the next tick (among those whose fields are ready)."""
        ready = self._ready()
        if self.tick_points is None:
            return ready
        chosen, total = [], 0
        for job in sorted(ready, key=lambda j: ((j.steps - j.done) * j.points, j.ident)):
            if chosen and total >= self.tick_points:
                break
            chosen.append(job)
            total += job.points
        return chosen

    def tick(self):
        """Issue ticks of the selected jobs; returns (the plans used, the jobs whose last step was issued).

        The selection cannot change before one of its jobs finishes (only selected jobs make progress, and
        arrivals are admitted between calls), so while it holds, up to ``BURST`` ticks of at most
        4 x ``tick_points`` points in all are issued at once: each is two launches of cached plans."""
        stepping = self.select()
        if not stepping:
            return [], []
        groups = {}
        for job in stepping:
            groups.setdefault(job.nscalar, []).append(job)
        points = sum(job.points for job in stepping)
        budget = 4 * (self.tick_points or points)
        burst = max(1, min(BURST, min(job.steps - job.done for job in stepping), budget // max(points, 1)))
        s = self.stream.cuda_stream
        used = []
        for _ in range(burst):
            for nscalar, jobs in sorted(groups.items()):
                plan = self._plan(nscalar, jobs)
                plan[0].step(s)
                plan[0].halo(s)
                used.append(plan)
                self.launches += 2
            for job in stepping:
                job.done += 1
            self.ticks += 1
        finishing = [job for job in stepping if job.done >= job.steps]
        return used, finishing

    # -- the open-loop run ------------------------------------------------------------------------
    def run(self, jobs: list[Job]) -> dict:
        torch = self.torch
        pending = sorted(jobs, key=lambda j: j.arrival)
        waiting: list[Job] = []
        start = time.perf_counter()
        i = 0
        finished = []

        def drain(block: bool) -> None:
            # retire the jobs of completed ticks, oldest first; `block` waits for the oldest one
            while self.inflight:
                event, _, done = self.inflight[0]
                if block:
                    event.synchronize()
                    block = False
                elif not event.query():
                    return
                now = time.perf_counter() - start
                for job in done:
                    self._retire(job, now)
                    finished.append(job)
                self.inflight.pop(0)

        while i < len(pending) or waiting or self.active or self.inflight:
            now = time.perf_counter() - start
            while i < len(pending) and pending[i].arrival <= now:
                waiting.append(pending[i])
                i += 1
            while waiting and self.fits(waiting[0]):
                self._admit(waiting.pop(0), now)
            if not self.active:
                if self.inflight:
                    drain(True)
                    continue
                if i < len(pending):  # idle until the next arrival
                    delay = pending[i].arrival - (time.perf_counter() - start)
                    if delay > 0:
                        time.sleep(delay)
                    continue
                if waiting:
                    raise RuntimeError("a job does not fit the device budget on its own")
                break
            if len(self.inflight) >= self.depth:
                drain(True)
            if not any(job.ready is None or job.ready.query() for job in self.active):
                # every active job is still being admitted: wait for the first of them
                next(job for job in self.active).ready.synchronize()
                continue
            used, done = self.tick()
            event = torch.cuda.Event()
            event.record(self.stream)
            self.inflight.append((event, used, done))
            if done:
                self.active = [j for j in self.active if j.done < j.steps]
            drain(False)
        wall = time.perf_counter() - start
        out = summarise(finished, wall, self.ticks, self.launches)
        out["plan_builds"] = self.plan_builds
        return out


class SerialServer:
    """The same open-loop stream served one job at a time through the single-instance path.

    A job is admitted when the previous one has finished (and it has arrived): its fields are generated on the
    device as the continuous server does, each step is one advection launch and one boundary fill, and the job
    is retired (one value read back) when its last step completes. Wall-clock, like ``Server.run``.
    """

    def __init__(self, torch):
        self.torch = torch
        self.stream = torch.cuda.Stream()
        self.launches = 0

    def run(self, jobs: list[Job]) -> dict:
        torch = self.torch
        start = time.perf_counter()
        finished = []
        for job in sorted(jobs, key=lambda j: j.arrival):
            delay = job.arrival - (time.perf_counter() - start)
            if delay > 0:
                time.sleep(delay)
            geo = job.geometry
            with torch.cuda.stream(self.stream):
                a = wl.advection_fields_device(geo, job.seed, job.nscalar, torch)
                b = [torch.empty_like(t) for t in a]
            grid = native.make_grid(geo.nx, geo.ny, geo.nz, geo.halo, geo.dx, geo.dy, geo.dz)
            kinds = [0, 0, 1] + [0] * job.nscalar
            s = self.stream.cuda_stream
            native.halo_fill(grid, [t.data_ptr() for t in a], kinds, stream=s)
            job.admitted = time.perf_counter() - start
            bufs = [a, b]
            for n in range(job.steps):
                src, dst = bufs[n % 2], bufs[1 - n % 2]
                p, q = [t.data_ptr() for t in src], [t.data_ptr() for t in dst]
                native.advection(grid, *p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:], mode=native.ADVANCE,
                                 dt=DT, stream=s)
                native.halo_fill(grid, q, kinds, stream=s)
            self.launches += 1 + 2 * job.steps
            with torch.cuda.stream(self.stream):
                bufs[job.steps % 2][0].view(-1)[:1].cpu()
            job.finished = time.perf_counter() - start
            finished.append(job)
        wall = time.perf_counter() - start
        return summarise(finished, wall, 0, self.launches)


def summarise(jobs: list[Job], wall: float, ticks: int = 0, launches: int = 0) -> dict:
    lat = np.array([(j.finished - j.arrival) * 1e3 for j in jobs])
    points = sum(j.points * j.steps for j in jobs)
    return {"jobs": len(jobs), "wall_s": wall, "jobs_per_s": len(jobs) / wall if wall > 0 else 0.0,
            "gpts_per_s": points / wall / 1e9 if wall > 0 else 0.0,
            "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
            "ticks": ticks, "launches": launches}


def solo_seconds(torch, job: Job) -> float:
    """Device time of one job run alone through the single-instance path (direct launches, one stream)."""
    geo = job.geometry
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        a = wl.advection_fields_device(geo, job.seed, job.nscalar, torch)
        b = [torch.empty_like(t) for t in a]
    grid = native.make_grid(geo.nx, geo.ny, geo.nz, geo.halo, geo.dx, geo.dy, geo.dz)
    kinds = [0, 0, 1] + [0] * job.nscalar
    native.halo_fill(grid, [t.data_ptr() for t in a], kinds, stream=stream.cuda_stream)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream.synchronize()
    start.record(stream)
    bufs = [a, b]
    for n in range(job.steps):
        src, dst = bufs[n % 2], bufs[1 - n % 2]
        p, q = [t.data_ptr() for t in src], [t.data_ptr() for t in dst]
        native.advection(grid, *p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:], mode=native.ADVANCE, dt=DT,
                         stream=stream.cuda_stream)
        native.halo_fill(grid, q, kinds, stream=stream.cuda_stream)
    stop.record(stream)
    stream.synchronize()
    return start.elapsed_time(stop) * 1e-3


def serial_timeline(jobs: list[Job], solo: dict) -> dict:
    """The stream served one job at a time (FIFO): start = max(arrival, previous finish)."""
    t = 0.0
    out = []
    for job in sorted(jobs, key=lambda j: j.arrival):
        begin = max(t, job.arrival)
        t = begin + solo[job.ident]
        out.append(Job(job.ident, job.arrival, job.nx, job.ny, job.nz, job.nscalar, job.steps, job.seed,
                       finished=t))
    return summarise(out, t)


def bench_main(args) -> None:
    """``bench.py --workload serving``: rates swept over {50, ..., 2000} jobs/s; continuous batching vs serial.

    Both servers run the same open-loop stream in wall-clock time with the same per-job work (fields generated
    on the device at admission, one value read back at retirement); ``serial_device_model`` adds the
    device-time-only FIFO model of the serial server (no host work at all) for reference.
    """
    import json

    import torch

    rates = (50, 100, 200, 500, 1000, 2000)
    count = max(20, getattr(args, "jobs", 50))
    # untimed warm-up of both servers (module loading, first allocations, plan building)
    Server(torch).run(poisson_jobs(8, 2000.0, seed=1))
    SerialServer(torch).run(poisson_jobs(8, 2000.0, seed=1))
    torch.cuda.synchronize()
    results = []
    for rate in rates:
        served = Server(torch).run(poisson_jobs(count, rate, seed=int(rate)))
        torch.cuda.synchronize()
        every = Server(torch, tick_points=None).run(poisson_jobs(count, rate, seed=int(rate)))
        torch.cuda.synchronize()
        serial = SerialServer(torch).run(poisson_jobs(count, rate, seed=int(rate)))
        torch.cuda.synchronize()
        jobs = poisson_jobs(count, rate, seed=int(rate))
        model = serial_timeline(jobs, {j.ident: solo_seconds(torch, j) for j in jobs})
        results.append({"rate_jobs_per_s": rate, "continuous_batching": served, "every_job_every_tick": every,
                        "serial_plain": serial,
                         "serial_device_model": model,
                         "throughput_ratio": served["gpts_per_s"] / serial["gpts_per_s"] if serial["gpts_per_s"]
                         else None,
                         "p99_ratio": served["p99_ms"] / serial["p99_ms"] if serial["p99_ms"] else None})
        torch.cuda.empty_cache()
    print(json.dumps({"metric": "serving: jobs/s, Gpts/s and p50/p99 job latency (continuous batching vs serial)",
                      "unit": "Gpts/s", "jobs_per_rate": count, "dtype": "f64",
                      "config": {"workload": "Poisson arrivals; nx,ny log-uniform [48,320] (independent draws), "
                                             "nz log-uniform [24,128], 0-3 scalars, 1-100 Euler steps",
                                 "budget_bytes": BUDGET_BYTES,
                                 "policy": f"shortest remaining work first, {TICK_POINTS} points per tick"},
                      "results": results}), flush=True)


__all__ = ["Job", "Server", "SerialServer", "poisson_jobs", "serial_timeline", "solo_seconds", "bench_main", "summarise"]
