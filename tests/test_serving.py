"""Serving: the arrival sampler and the serial timeline (CPU), continuous batching results (GPU)."""

import numpy as np
import pytest

from compiler import serving


def test_poisson_stream_is_seeded_and_in_range():
    jobs = serving.poisson_jobs(400, rate=200.0, seed=3)
    assert [j.arrival for j in jobs] == [j.arrival for j in serving.poisson_jobs(400, rate=200.0, seed=3)]
    gaps = np.diff([0.0] + [j.arrival for j in jobs])
    assert (gaps > 0).all() and abs(gaps.mean() - 1 / 200.0) < 0.25 / 200.0
    assert all(48 <= j.nx <= 320 and 48 <= j.ny <= 320 and 24 <= j.nz <= 128 for j in jobs)
    assert {j.nscalar for j in jobs} == {0, 1, 2, 3}
    assert min(j.steps for j in jobs) >= 1 and max(j.steps for j in jobs) <= 100
    # log-uniform: the median size is near the geometric mean of the range
    assert 100 < np.median([j.nx for j in jobs]) < 150


def test_serial_timeline_is_fifo():
    jobs = [serving.Job(n, arrival=a, nx=48, ny=48, nz=24, nscalar=0, steps=1, seed=n)
            for n, a in enumerate([0.0, 0.1, 0.15, 1.0])]
    solo = {0: 0.2, 1: 0.2, 2: 0.1, 3: 0.05}
    out = serving.serial_timeline(jobs, solo)
    # finishes: 0.2, 0.4, 0.5, 1.05; latencies 0.2, 0.3, 0.35, 0.05 s
    assert out["jobs"] == 4
    assert abs(out["wall_s"] - 1.05) < 1e-12
    assert abs(out["p50_ms"] - 250.0) < 1e-6


def _mix():
    shapes = [(48, 52, 24, 0, 3), (70, 49, 31, 1, 5), (96, 64, 26, 3, 2), (51, 90, 40, 2, 4), (64, 64, 24, 1, 1)]
    return [serving.Job(n, arrival=0.002 * n, nx=a, ny=b, nz=c, nscalar=s, steps=t, seed=500 + n)
            for n, (a, b, c, s, t) in enumerate(shapes)]


@pytest.mark.gpu
def test_each_job_is_the_same_alone_and_in_the_mix(cuda):
    from compiler import workloads as wl
    from oracle import api

    jobs = _mix()
    summary = serving.Server(cuda, keep_results=True).run(jobs)
    assert summary["jobs"] == len(jobs) and summary["ticks"] >= max(j.steps for j in jobs)
    in_mix = {j.ident: j.result for j in jobs}
    for job in _mix():
        one = serving.Job(job.ident, 0.0, job.nx, job.ny, job.nz, job.nscalar, job.steps, job.seed)
        serving.Server(cuda, keep_results=True).run([one])
        assert len(one.result) == 3 + job.nscalar
        for a, b in zip(in_mix[job.ident], one.result):
            assert np.array_equal(a.view(np.int64), b.view(np.int64))
    # one job against the oracle: its initial fields with the boundary fill, then Euler steps with the fill
    job = _mix()[1]
    geo = job.geometry
    init = [t.cpu().numpy() for t in wl.advection_fields_device(geo, job.seed, job.nscalar, cuda)]
    state = [api.halo(x.copy(), 1 if n == 2 else 0, geo.halo) for n, x in enumerate(init)]
    names = ["U", "V", "W", *[f"S{n}" for n in range(job.nscalar)]]
    for _ in range(job.steps):
        t = api.advection_step({"U": state[0], "V": state[1], "W": state[2]}, geo.dx, geo.dy, geo.dz, geo.halo,
                               state[3:])
        new = [api.euler(x.copy(), t[name], serving.DT, geo.halo) for x, name in zip(state, names)]
        state = [api.halo(x, 1 if n == 2 else 0, geo.halo) for n, x in enumerate(new)]
    for got, want in zip(in_mix[job.ident], state):
        assert np.array_equal(got.view(np.int64), want.view(np.int64))


def test_tick_selection_takes_shortest_remaining_work_first():
    class Stub(serving.Server):
        def __init__(self, tick_points):  # no device: only the selection rule
            self.tick_points = tick_points
            self.active = []

    jobs = [serving.Job(n, 0.0, nx, 100, 10, 0, steps, seed=n)
            for n, (nx, steps) in enumerate([(100, 50), (100, 5), (200, 5), (100, 6)])]
    jobs[0].done = 48  # 2 steps left
    server = Stub(tick_points=250_000)
    server.active = jobs
    # remaining work: job0 2x1e5, job1 5x1e5, job3 6x1e5, job2 5x2e5: the first three fill 3e5 >= 2.5e5 points
    assert [j.ident for j in server.select()] == [0, 1, 3]
    server.tick_points = None
    assert [j.ident for j in server.select()] == [0, 1, 2, 3]
    server.tick_points = 1
    assert [j.ident for j in server.select()] == [0]  # always at least one job


def test_tick_chunk_depth_spreads_small_ticks():
    assert serving.tick_chunk_depth([(512, 512, 128)] * 4, 152) == 32
    # one 64x64x32 job: 16 column tiles x 32 levels = 512 tile-levels over 608 CTAs: the shallowest chunks
    assert serving.tick_chunk_depth([(64, 64, 32)], 152) == 2
    assert serving.tick_chunk_depth([(160, 160, 64)], 152) == 11  # 100 tiles x 64 levels / 608
