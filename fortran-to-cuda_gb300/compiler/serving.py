"""Serving advection jobs with continuous batching.

A job asks for ``steps`` forward-Euler steps (dt = 0.1, with the boundary fill
after each) of an advection instance: seeded sine-mode U, V, W and 0-3
scalars on an nx x ny x nz grid. ``Server`` drives the native server of
``include/f2c_serve.h``: a worker thread in the library admits jobs as they
arrive while free device memory covers them, keeps each job's two field sets
in the residency runtime's device mirrors from admission to retirement (its
first set seeded on the device, nothing moved to the host between steps), and
advances the jobs with the least remaining work, up to about 8 M grid points a
tick, as one persistent batched launch per scalar count that also fills the
new fields' ghost layers, two ticks of a selection captured once as a CUDA
graph and replayed while the selection holds. Every job's arithmetic is the
single-instance kernel's, so a job's result is the same alone and in any mix,
bit for bit.

The open-loop arrival stream and the job sizes follow the serving
configuration: Poisson arrivals at a given rate; nx and ny drawn independently
log-uniform in [48, 320], nz log-uniform in [24, 128]; 0-3 scalars and 1-100
steps uniform. ``SerialServer`` gives the comparison: the same stream served
one job at a time through the single-instance path, in wall-clock time with
the same per-job work; ``serial_timeline`` models it from device times alone.
"""

from __future__ import annotations

import ctypes
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import native
from . import workloads as wl

DT = 0.1
BUDGET_BYTES = 150 * 10**9
MAX_ACTIVE = 256
# grid points advanced per tick before further jobs wait for the next tick: about 1.3 ms of fast-fp work. Measured
# on GB300 (500 jobs at 200 and 2000 jobs/s): 4 M-point ticks gave 1.04-1.06x the device-time model of serial
# service with a median latency of 86 ms at 200 jobs/s, 8 M 1.07-1.09x and 135 ms, 16 M 1.09-1.11x and 231 ms
TICK_POINTS = 8_000_000
# jobs waiting longer than this since their arrival go first, oldest first. Measured on GB300 (500 jobs at 200
# jobs/s): 2 s keeps the throughput (6.54 Gpts/s) and nearly the median latency (130 ms against 91 ms for
# least remaining work alone) and cuts the p99 from 4.1 s to 2.4 s; 0.5-1 s makes most jobs old and the median
# rises to 1.5 s. At 2000 jobs/s the backlog is so deep that no setting changes the p99 (4.4-4.6 s).
STARVE_S = 2.0
NUMERICS = {"fast": native.FAST, "strict": native.FACES}


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
    admitted: float = -1.0
    finished: float = -1.0
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


class ServeError(RuntimeError):
    pass


class Server:
    """Continuous batching through the native server, on a residency domain of its own.

    ``numerics`` is the domain's numerical contract ("fast": the fast-fp kernels, "strict": bit-identical to the
    oracle). ``tick_points=None`` steps every resident job every tick. ``graphs=False`` launches ticks directly.
    ``keep_results`` publishes every job's final fields into ``Job.result`` (numpy arrays, padded layout).
    ``reserve_bytes`` is the device memory every admission leaves free (0: max(total/16, 512 MiB)).
    ``starve_s`` > 0 lets jobs that have waited that long since their arrival go first, oldest first.
    """

    def __init__(self, torch=None, numerics: str = "fast", budget_bytes: int = BUDGET_BYTES,
                 max_active: int = MAX_ACTIVE, keep_results: bool = False, depth: int = 4,
                 tick_points: int | None = TICK_POINTS, graphs: bool = True, device: int = 0,
                 reserve_bytes: int = 0, starve_s: float = STARVE_S):
        self.numerics = numerics
        self.reserve = reserve_bytes
        self.starve_s = starve_s
        self.budget = budget_bytes
        self.max_active = max_active
        self.keep_results = keep_results
        self.depth = depth
        self.tick_points = tick_points
        self.graphs = graphs
        self.device = device
        self.stats = {}

    def run(self, jobs: list[Job]) -> dict:
        from .resident.domain import ResidentDomain

        lib = native.runtime()
        dom = ResidentDomain(lib, fast_fp=self.numerics == "fast")
        dom.begin_epoch(device=self.device)
        # the jobs' arrays never move between host and device while in use: no pinning
        dom.require(lib.fort_scope_host_pinning_set_v1(dom.context, 0))
        opts = native.ServeOptions(version=native.SERVE_ABI_VERSION, flags=0 if self.graphs else native.SERVE_DIRECT,
                                   max_active=self.max_active, depth=self.depth, budget_bytes=self.budget,
                                   reserve_bytes=self.reserve, tick_points=self.tick_points or (1 << 62),
                                   burst_points=0, starve_s=self.starve_s)
        handle = ctypes.c_uint64()
        self._check(lib.f2c_serve_create_v1(dom.context, ctypes.byref(opts), ctypes.byref(handle)), 0)
        server = handle.value
        try:
            return self._serve(lib, server, jobs)
        finally:
            lib.f2c_serve_destroy_v1(server)
            dom.close()

    def _check(self, status: int, server: int) -> None:
        if status != 0:
            lib = native.load()
            text = lib.f2c_serve_error_v1(server) if server else native.runtime().fort_scope_error()
            raise ServeError(f"server status {status}: {text.decode(errors='replace')}")

    def _serve(self, lib, server: int, jobs: list[Job]) -> dict:
        ordered = sorted(jobs, key=lambda j: j.arrival)
        start = lib.f2c_serve_clock_v1(server) + 0.01  # the stream starts once every job is queued
        by_id = {}
        for job in ordered:
            g = job.geometry
            spec = native.ServeJob(nx=g.nx, ny=g.ny, nz=g.nz, halo=g.halo, dx=g.dx, dy=g.dy, dz=g.dz, dt=DT,
                                   nscalar=job.nscalar, steps=job.steps, seed=job.seed,
                                   arrival=start + job.arrival,
                                   flags=native.SERVE_KEEP_RESULT if self.keep_results else 0, reserved=0)
            ident = ctypes.c_uint64()
            self._check(lib.f2c_serve_submit_v1(server, ctypes.byref(spec), ctypes.byref(ident)), server)
            by_id[ident.value] = job
        self._check(lib.f2c_serve_drain_v1(server, -1.0), server)
        records = (native.ServeDone * max(1, len(ordered)))()
        count = ctypes.c_size_t()
        self._check(lib.f2c_serve_poll_v1(server, records, len(ordered), ctypes.byref(count)), server)
        finished = []
        for r in records[:count.value]:
            job = by_id[r.id]
            if r.status != 0:
                raise ServeError(f"job {job.ident} failed with status {r.status}")
            job.admitted, job.finished = r.admitted - start, r.finished - start
            finished.append(job)
            if self.keep_results:
                shape = job.geometry.shape
                out = []
                for f in range(3 + job.nscalar):
                    ptr = ctypes.POINTER(ctypes.c_double)()
                    self._check(lib.f2c_serve_result_v1(server, r.id, f, ctypes.byref(ptr)), server)
                    out.append(np.ctypeslib.as_array(ptr, shape=shape).copy())
                job.result = out
                self._check(lib.f2c_serve_release_v1(server, r.id), server)
        stats = native.ServeStats()
        self._check(lib.f2c_serve_stats_get_v1(server, ctypes.byref(stats)), server)
        self.stats = stats.as_dict()
        wall = max((j.finished for j in finished), default=0.0)
        out = summarise(finished, wall, stats.ticks, stats.graph_replays + stats.direct_launches)
        out["server"] = self.stats
        return out


def _device_job(torch, job: Job, stream):
    """A job's two field sets as torch tensors, the first seeded on the device (as the server seeds it)."""
    geo = job.geometry
    with torch.cuda.stream(stream):
        a = [torch.empty(geo.shape, dtype=torch.float64, device="cuda") for _ in range(3 + job.nscalar)]
        b = [torch.empty_like(t) for t in a]
    grid = native.make_grid(geo.nx, geo.ny, geo.nz, geo.halo, geo.dx, geo.dy, geo.dz)
    native.seed_fields(grid, job.seed, [t.data_ptr() for t in a], stream=stream.cuda_stream)
    return grid, [a, b]


def _plain_steps(grid, bufs, job: Job, variant: int, stream: int) -> None:
    """The job's steps through the single-instance path: one launch per step (advance and boundary fill)."""
    for n in range(job.steps):
        src, dst = bufs[n % 2], bufs[1 - n % 2]
        p, q = [t.data_ptr() for t in src], [t.data_ptr() for t in dst]
        native.advection(grid, *p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:], mode=native.ADVANCE_FILLED, dt=DT,
                         stream=stream, variant=variant)


class SerialServer:
    """The same open-loop stream served one job at a time through the single-instance path.

    A job is admitted when the previous one has finished (and it has arrived): its fields are seeded on the
    device as the continuous server seeds them, each step is one advection launch that also fills the boundary,
    and the job is retired (one value read back) when its last step completes. Wall-clock, like ``Server.run``.
    """

    def __init__(self, torch, numerics: str = "fast"):
        self.torch = torch
        self.variant = NUMERICS[numerics]
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
            job.admitted = time.perf_counter() - start
            grid, bufs = _device_job(torch, job, self.stream)
            _plain_steps(grid, bufs, job, self.variant, self.stream.cuda_stream)
            self.launches += 2 + job.steps
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


def solo_seconds(torch, job: Job, numerics: str = "fast") -> float:
    """Device time of one job run alone through the single-instance path (direct launches, one stream)."""
    stream = torch.cuda.Stream()
    grid, bufs = _device_job(torch, job, stream)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream.synchronize()
    start.record(stream)
    _plain_steps(grid, bufs, job, NUMERICS[numerics], stream.cuda_stream)
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


def measure_rate(torch, rate: float, count: int, numerics: str = "fast", every_tick: bool = False) -> dict:
    """One rate: continuous batching, the serial server and the device-time model of serial service."""
    served = Server(torch, numerics=numerics).run(poisson_jobs(count, rate, seed=int(rate)))
    torch.cuda.synchronize()
    out = {"rate_jobs_per_s": rate, "jobs": count, "continuous_batching": served}
    if every_tick:
        out["every_job_every_tick"] = Server(torch, numerics=numerics, tick_points=None).run(
            poisson_jobs(count, rate, seed=int(rate)))
    serial = SerialServer(torch, numerics).run(poisson_jobs(count, rate, seed=int(rate)))
    torch.cuda.synchronize()
    jobs = poisson_jobs(count, rate, seed=int(rate))
    model = serial_timeline(jobs, {j.ident: solo_seconds(torch, j, numerics) for j in jobs})
    torch.cuda.empty_cache()
    out.update({"serial_plain": serial, "serial_device_model": model,
                "throughput_ratio": served["gpts_per_s"] / serial["gpts_per_s"] if serial["gpts_per_s"] else None,
                "over_device_model": served["gpts_per_s"] / model["gpts_per_s"] if model["gpts_per_s"] else None,
                "p99_ratio": served["p99_ms"] / serial["p99_ms"] if serial["p99_ms"] else None})
    return out


def warm_up(torch, numerics: str = "fast") -> None:
    """Untimed first use of both servers (module loading, first allocations)."""
    Server(torch, numerics=numerics).run(poisson_jobs(8, 2000.0, seed=1))
    SerialServer(torch, numerics).run(poisson_jobs(8, 2000.0, seed=1))
    torch.cuda.synchronize()


def bench_main(args) -> None:
    """``bench.py --workload serving``: rates swept over {50, ..., 2000} jobs/s; continuous batching vs serial."""
    import json

    import torch

    rates = tuple(getattr(args, "rates", None) or (50, 100, 200, 500, 1000, 2000))
    count = max(20, getattr(args, "jobs", 500))
    numerics = getattr(args, "numerics", "fast")
    warm_up(torch, numerics)
    results = [measure_rate(torch, rate, count, numerics, every_tick=True) for rate in rates]
    print(json.dumps({"metric": "serving: jobs/s, Gpts/s and p50/p99 job latency (continuous batching vs serial)",
                      "unit": "Gpts/s", "jobs_per_rate": count, "dtype": "f64", "numerics": numerics,
                      "config": config(), "results": results}), flush=True)


def config() -> dict:
    return {"workload": "Poisson arrivals; nx,ny log-uniform [48,320] (independent draws), nz log-uniform [24,128], "
                        "0-3 scalars, 1-100 Euler steps, fields seeded on the device",
            "budget_bytes": BUDGET_BYTES,
            "policy": f"least remaining work first (jobs older than {STARVE_S} s first, oldest first), "
                      f"{TICK_POINTS} points per tick, two-tick graphs"}


__all__ = ["Job", "Server", "SerialServer", "poisson_jobs", "serial_timeline", "solo_seconds", "bench_main",
           "summarise", "measure_rate", "warm_up", "config"]
