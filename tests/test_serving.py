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


def _same(a, b):
    return all(np.array_equal(x.view(np.int64), y.view(np.int64)) for x, y in zip(a, b, strict=True))


def _seeded(cuda, job):
    from compiler import native

    geo = job.geometry
    fields = [cuda.empty(geo.shape, dtype=cuda.float64, device="cuda") for _ in range(3 + job.nscalar)]
    grid = native.make_grid(geo.nx, geo.ny, geo.nz, geo.halo, geo.dx, geo.dy, geo.dz)
    native.seed_fields(grid, job.seed, [t.data_ptr() for t in fields])
    cuda.cuda.synchronize()
    return [t.cpu().numpy() for t in fields]


def _oracle_run(job, init):
    from oracle import api

    geo = job.geometry
    state = [x.copy() for x in init]
    names = ["U", "V", "W", *[f"S{n}" for n in range(job.nscalar)]]
    for _ in range(job.steps):
        t = api.advection_step({"U": state[0], "V": state[1], "W": state[2]}, geo.dx, geo.dy, geo.dz, geo.halo,
                               state[3:])
        new = [api.euler(x.copy(), t[name], serving.DT, geo.halo) for x, name in zip(state, names)]
        state = [api.halo(x, 1 if n == 2 else 0, geo.halo) for n, x in enumerate(new)]
    return state


@pytest.mark.gpu
@pytest.mark.parametrize("numerics", ["strict", "fast"])
def test_each_job_is_the_same_alone_and_in_the_mix(cuda, numerics):
    jobs = _mix()
    server = serving.Server(cuda, numerics=numerics, keep_results=True)
    summary = server.run(jobs)
    assert summary["jobs"] == len(jobs) and summary["ticks"] >= max(j.steps for j in jobs)
    in_mix = {j.ident: j.result for j in jobs}
    for job in _mix():
        one = serving.Job(job.ident, 0.0, job.nx, job.ny, job.nz, job.nscalar, job.steps, job.seed)
        serving.Server(cuda, numerics=numerics, keep_results=True).run([one])
        assert len(one.result) == 3 + job.nscalar
        assert _same(in_mix[job.ident], one.result)
    # every job against the oracle: its seeded fields, then Euler steps with the boundary fill
    from tolerance import check

    for job in _mix():
        want = _oracle_run(job, _seeded(cuda, job))
        inner = job.geometry.interior()
        for n, (got, ref) in enumerate(zip(in_mix[job.ident], want)):
            if numerics == "strict":
                assert np.array_equal(got.view(np.int64), ref.view(np.int64)), (job.ident, n)
            else:
                check(got[inner], ref[inner], f"job {job.ident} field {n}")


@pytest.mark.gpu
def test_graph_replay_equals_direct_launches(cuda):
    jobs = serving.poisson_jobs(12, rate=5000.0, seed=7)
    graphed = serving.Server(cuda, keep_results=True)
    graphed.run(jobs)
    assert graphed.stats["graph_replays"] > 0 and graphed.stats["direct_launches"] == 0
    assert graphed.stats["graph_builds"] <= graphed.stats["graph_replays"]
    again = serving.poisson_jobs(12, rate=5000.0, seed=7)
    direct = serving.Server(cuda, keep_results=True, graphs=False)
    direct.run(again)
    assert direct.stats["graph_replays"] == 0 and direct.stats["direct_launches"] > 0
    for a, b in zip(jobs, again):
        assert _same(a.result, b.result)


@pytest.mark.gpu
def test_admission_waits_for_device_budget(cuda):
    jobs = [serving.Job(n, 0.0, 96, 96, 48, 1, 3, seed=900 + n) for n in range(6)]
    per_job = jobs[0].device_bytes()
    server = serving.Server(cuda, keep_results=True, budget_bytes=2 * per_job + per_job // 2)
    summary = server.run(jobs)
    assert summary["jobs"] == 6
    # never more than two jobs resident; the others waited for retirements
    assert server.stats["peak_job_bytes"] <= 2 * per_job and server.stats["peak_active"] <= 2
    assert server.stats["refused_admissions"] > 0
    alone = serving.Job(3, 0.0, 96, 96, 48, 1, 3, seed=903)
    serving.Server(cuda, keep_results=True).run([alone])
    assert _same(jobs[3].result, alone.result)


@pytest.mark.gpu
def test_a_job_larger_than_the_budget_fails_alone(cuda):
    big = serving.Job(0, 0.0, 64, 64, 32, 0, 2, seed=1)
    with pytest.raises(serving.ServeError, match="status 4"):
        serving.Server(cuda, budget_bytes=big.device_bytes() // 2).run([big])


@pytest.mark.gpu
def test_seeded_fields_follow_the_recipe(cuda):
    """The device generator against a numpy restatement of its recipe (counter-based draws, sine modes)."""
    from compiler import workloads as wl

    job = serving.Job(0, 0.0, 40, 24, 12, 4, 1, seed=12345)
    got = _seeded(cuda, job)
    want = wl.seeded_fields_reference(job.geometry, job.seed, job.nscalar)
    inner = job.geometry.interior()
    for n, (g, w) in enumerate(zip(got, want)):
        if n in (3, 4):  # the uniform scalars: 53-bit draws, exact
            assert np.array_equal(g[inner], w[inner])
        else:  # single-precision sin, cos, log and exp may differ by a few units in a float's last place
            assert np.allclose(g[inner], w[inner], rtol=0, atol=2e-5)
    # deterministic, ghosts filled as the boundary rule says
    assert _same(got, _seeded(cuda, job))
    from oracle import api

    for n, g in enumerate(got):
        assert np.array_equal(g, api.halo(g.copy(), 1 if n == 2 else 0, job.geometry.halo))
    # the noise is N(0, 0.05) and the first scalar uniform in [280, 300]
    assert 280.0 <= got[3][inner].min() and got[3][inner].max() <= 300.0


@pytest.mark.gpu
def test_admission_follows_free_device_memory(cuda):
    """With the reserve set so that the device's free memory covers two jobs, at most two are resident."""
    jobs = [serving.Job(n, 0.0, 128, 120, 64, 2, 4, seed=700 + n) for n in range(5)]
    per_job = jobs[0].device_bytes()
    cuda.cuda.synchronize()
    free, _ = cuda.cuda.mem_get_info()
    # the server's own plan slots (64 MiB) come out of free memory too
    server = serving.Server(cuda, keep_results=True, reserve_bytes=free - (64 << 20) - int(2.5 * per_job))
    summary = server.run(jobs)
    assert summary["jobs"] == 5
    assert server.stats["peak_active"] <= 2 and server.stats["refused_admissions"] > 0
    alone = serving.Job(4, 0.0, 128, 120, 64, 2, 4, seed=704)
    serving.Server(cuda, keep_results=True).run([alone])
    assert _same(jobs[4].result, alone.result)


@pytest.mark.gpu
def test_no_free_memory_refuses_the_job(cuda):
    job = serving.Job(0, 0.0, 48, 48, 24, 0, 1, seed=3)
    free, total = cuda.cuda.mem_get_info()
    with pytest.raises(serving.ServeError, match="status 4"):
        serving.Server(cuda, reserve_bytes=total).run([job])


@pytest.mark.gpu
@pytest.mark.parametrize("numerics", ["fast", "strict"])
def test_a_poisson_mix_equals_one_job_at_a_time(cuda, numerics):
    """24 jobs of the serving distribution through continuous batching, each bit-identical to the same job run
    alone through the single-instance path (seeded alike, one filled-advance launch per step)."""
    jobs = serving.poisson_jobs(24, rate=3000.0, seed=77)
    for job in jobs:  # keep the test short: at most 12 steps per job
        job.steps = 1 + job.steps % 12
    served = serving.Server(cuda, numerics=numerics, keep_results=True, tick_points=3_000_000)
    served.run(jobs)
    assert served.stats["graph_replays"] > 0
    stream = cuda.cuda.Stream()
    for job in jobs:
        grid, bufs = serving._device_job(cuda, job, stream)
        serving._plain_steps(grid, bufs, job, serving.NUMERICS[numerics], stream.cuda_stream)
        stream.synchronize()
        alone = [t.cpu().numpy() for t in bufs[job.steps % 2]]
        assert _same(job.result, alone), job.ident


@pytest.mark.gpu
def test_edge_sized_jobs_and_four_scalars(cuda):
    """Jobs at the smallest grids the boundary rule allows (nx = ny = halo, nz = halo + 1), with four scalars,
    mixed with ordinary ones: each equals the same job alone."""
    shapes = [(2, 2, 3, 4, 3), (2, 5, 3, 0, 2), (33, 2, 4, 4, 5), (70, 41, 29, 4, 4), (64, 64, 24, 1, 6)]
    jobs = [serving.Job(n, 0.001 * n, a, b, c, s, t, seed=900 + n) for n, (a, b, c, s, t) in enumerate(shapes)]
    serving.Server(cuda, keep_results=True).run(jobs)
    stream = cuda.cuda.Stream()
    for job in jobs:
        grid, bufs = serving._device_job(cuda, job, stream)
        serving._plain_steps(grid, bufs, job, serving.NUMERICS["fast"], stream.cuda_stream)
        stream.synchronize()
        assert _same(job.result, [t.cpu().numpy() for t in bufs[job.steps % 2]]), job.ident
