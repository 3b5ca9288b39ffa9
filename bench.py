"""Headline benchmark of the GB300 resident advection path.

Workload (the reference's headline configuration that fits one GPU): the
advection step of the cdu driver restated on a 512 x 512 x 128 FP64 grid with
halo 2 and spacings 10/10/5 m, U, V, W from the seeded sine-mode recipe plus
three passive scalars; one step computes the U, V, W and scalar tendencies
(the cdu driver's semantics: benchmarks/cdu/src/main.f90:67-79 recomputes U2
from fixed fields every iteration). The step is captured once as a CUDA graph
and replayed. Inputs (12 arrays, 3.4 GB) exceed L2 (129 MB), so no flush is
needed between steps.

``python bench.py [--gpus N --steps K --warmup W]`` prints one JSON line.
``--impl reference`` times the CPU implementation of the same step (the C
oracle restating cdu.f90/cvd.f90/cdw.f90; the reference's own native control
needs a Fortran compiler that neither machine has) on all host cores.
Under torchrun each rank runs an independent replica (the path does not need a
data-path collective); value = all ranks' points x steps / slowest rank's time.
"""

from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path[:0] = [str(ROOT), str(ROOT / "fortran-to-cuda_gb300")]

NX, NY, NZ, HALO = 512, 512, 128, 2
DX, DY, DZ = 10.0, 10.0, 5.0
NSCALAR = 3
METRIC = "advection Gpts/s (512x512x128 FP64 U,V,W + 3 scalars tendency step, graph-replayed)"
UNIT = "Gpts/s"
FALLBACK_HBM_GBS = 6800.0


def algorithmic_bytes_per_point(nscalar: int, mode: str = "tendency") -> int:
    """Compulsory HBM bytes per interior point: each array read once and written once."""
    if mode == "tendency":
        return 8 * (3 + 3) + 16 * nscalar
    return 2 * (24 + 8 * nscalar)


def fp64_ops_per_point(nscalar: int) -> int:
    """FP64 operations per point with every face flux computed once (the minimum for these formulas).

    U, V, W: 9 face sums + 18 flux products + 15 flux differences + 51 advective-form operations
    (of which 3 are the exact halving); scalars: 3 shared coefficient products + 11 per scalar.
    """
    return 93 + (3 + 11 * nscalar if nscalar else 0)


def hbm_peak():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        data = json.loads(path.read_text())
        if data.get("hbm_gbs"):
            return float(data["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples taken while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.device_index = device_index
        self.proc = None
        self.file = None

    def __enter__(self):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device_index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        self.file.flush()
        return False

    def summary(self):
        try:
            text = Path(self.file.name).read_text()
            os.unlink(self.file.name)
        except OSError:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = [r for r in csv.reader(io.StringIO(text)) if len(r) >= 9]
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except ValueError:
                continue
            for name, flag in zip(names, r[5:9]):
                if flag.strip().lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": smax, "reasons": ["unsampled"]}
        busy = sorted(sm)[len(sm) // 2:] if len(sm) > 4 else sm
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl"
        dist.init_process_group(backend=backend)
        return dist, rank, world, local
    return None, rank, world, local


def barrier(dist, torch):
    if dist is not None:
        dist.barrier(device_ids=[torch.cuda.current_device()])


def max_over_ranks(dist, torch, value: float) -> float:
    if dist is None:
        return value
    t = torch.tensor([value], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_oracle_sample(fields, budget_s: float = 12.0):
    """Time the C oracle (all host threads) on the full workload; returns (Gpts/s, threads, sample text)."""
    from oracle import api

    geo = fields.geometry
    arrays = {"U": fields.U, "V": fields.V, "W": fields.W}
    out = api.advection_step(arrays, geo.dx, geo.dy, geo.dz, geo.halo, fields.scalars)  # warm-up
    times = []
    start = time.perf_counter()
    while not times or (time.perf_counter() - start < budget_s and len(times) < 5):
        t0 = time.perf_counter()
        api.advection_step(arrays, geo.dx, geo.dy, geo.dz, geo.halo, fields.scalars, out=out)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    return geo.points / t / 1e9, api.threads(), f"{len(times)} full steps (median) after 1 warm-up"


def run_e2e(fields, steps, dist, torch):
    """Gpts/s of the step through the residency runtime and the generated entry, host buffers in and out."""
    from compiler import emission, native
    from compiler.resident.domain import ResidentDomain
    from compiler.runtime import abi

    geo = fields.geometry
    lib = native.runtime()
    functions = emission.bind(lib)
    dom = ResidentDomain(lib)
    inputs = fields.arrays()
    outputs = [np.zeros_like(a) for a in inputs]
    dom.begin_epoch()
    h_in = [dom.bind_real64(a) for a in inputs]
    h_out = [dom.bind_real64(a) for a in outputs]
    arrays = [*h_out[:3], *h_in[:3], *h_in[3:], *h_out[3:]]
    grid = [geo.nx, geo.ny, geo.nz, geo.halo]
    entry = f"advection::step{len(inputs) - 3}"

    def step():
        dom.host_modify(h_in)
        status = emission.call(functions, entry, dom.context, abi.GPU, arrays, [geo.dx, geo.dy, geo.dz], grid)
        if status != abi.OK:
            raise RuntimeError(f"{entry} returned {status}: {lib.fort_scope_error().decode()}")
        dom.observe(h_out)

    for _ in range(2):
        step()
    n = max(1, min(steps, 5))
    barrier(dist, torch)
    t0 = time.perf_counter()
    for _ in range(n):
        step()
    elapsed = time.perf_counter() - t0
    elapsed = max_over_ranks(dist, torch, elapsed)
    dom.end_epoch()
    dom.close()
    world = dist.get_world_size() if dist is not None else 1
    nbytes = sum(a.nbytes for a in inputs)
    return geo.points * world * n / elapsed / 1e9, n, nbytes, sum(a.nbytes for a in outputs)


def run_gb300(args):
    import torch

    from compiler import native
    from compiler import workloads as wl

    dist, rank, world, local = dist_setup()
    torch.cuda.set_device(local)
    geo = wl.Geometry(NX, NY, NZ, halo=HALO, dx=DX, dy=DY, dz=DZ)
    fields = wl.advection_fields(geo, seed=rank, nscalar=NSCALAR)
    host_inputs = fields.arrays()
    dev_in = [torch.from_numpy(a).cuda() for a in host_inputs]
    dev_out = [torch.zeros_like(t) for t in dev_in]
    grid = native.make_grid(NX, NY, NZ, HALO, DX, DY, DZ)
    p = [t.data_ptr() for t in dev_in]
    q = [t.data_ptr() for t in dev_out]
    stream = torch.cuda.Stream()

    def launch(s):
        native.advection(grid, *p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:], stream=s)

    # one step captured as a CUDA graph, replayed
    with torch.cuda.stream(stream):
        launch(stream.cuda_stream)  # warm the module before capture
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        launch(stream.cuda_stream)
    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize()

    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as sampler:
        barrier(dist, torch)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            start.record(stream)
            for _ in range(args.steps):
                graph.replay()
            stop.record(stream)
        torch.cuda.synchronize()
        barrier(dist, torch)
    elapsed_ms = start.elapsed_time(stop)
    elapsed_ms = max_over_ranks(dist, torch, elapsed_ms)
    ms_per_step = elapsed_ms / args.steps
    points = geo.points
    value = points * world * args.steps / (elapsed_ms * 1e-3) / 1e9

    # FP64 pipe rate of this GPU (the roofline that binds first on GB300)
    scratch = torch.empty(8 * torch.cuda.get_device_properties(local).multi_processor_count * 256,
                          dtype=torch.float64, device="cuda")
    fp64_add = native.fp64_rate(0, scratch.data_ptr(), scratch.numel())
    fp64_fma = native.fp64_rate(1, scratch.data_ptr(), scratch.numel())
    del scratch

    # End to end through the reference-facing C ABI: a residency domain holds the host arrays (pinned in
    # place at registration), every step the host rewrites the inputs (their device copies go stale), the
    # generated entry advection::step3 runs (uploading what changed) and the outputs are published back.
    e2e_value, e2e_steps, bytes_in, bytes_out = run_e2e(fields, args.steps, dist, torch)

    peak, peak_kind = hbm_peak()
    alg = algorithmic_bytes_per_point(NSCALAR) * points
    achieved = alg / (ms_per_step * 1e-3) / 1e9
    traffic = None
    traffic_file = ROOT / "profiles" / "advection_512x512x128_s3_traffic.txt"
    if traffic_file.exists():
        for line in traffic_file.read_text().splitlines():
            if line.startswith("dram_bytes_per_launch"):
                traffic = float(line.split("=")[1])
    fp64_alg = fp64_ops_per_point(NSCALAR) * points / (ms_per_step * 1e-3)
    fp64_peak = max(fp64_add, fp64_fma)

    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded sine modes + noise, scalars)",
        "config": {"workload": "advection 512x512x128 halo 2 + 3 scalars, tendency step, CUDA graph replay",
                   "nx": NX, "ny": NY, "nz": NZ, "halo": HALO, "scalars": NSCALAR,
                   "parallelism": f"replicas x{world}", "l2": "inputs 3.4 GB > L2, no flush"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": f"{peak_kind} hbm_gbs",
                     "algorithmic_bytes_per_launch": alg},
        "fp64_roofline": {"achieved_ops_per_s": fp64_alg, "peak_ops_per_s": fp64_peak,
                          "frac": fp64_alg / fp64_peak, "ops_per_point": fp64_ops_per_point(NSCALAR),
                          "peak_add_rn": fp64_add, "peak_fma_rn": fp64_fma, "peak_source": "measured live"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": bytes_in,
                "d2h_bytes_per_step": bytes_out, "steps": e2e_steps,
                "path": "fort_scope runtime + generated entry advection::step3 (host arrays, upload/publish per step)"},
        "gpu_launches": args.steps,
        "clocks": sampler.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, sample = cpu_oracle_sample(fields)
        result["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
    if rank == 0:
        print(json.dumps(result), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from compiler import workloads as wl
    from oracle import api

    warmup = max(3, args.warmup)
    geo = wl.Geometry(NX, NY, NZ, halo=HALO, dx=DX, dy=DY, dz=DZ)
    fields = wl.advection_fields(geo, seed=0, nscalar=NSCALAR)
    arrays = {"U": fields.U, "V": fields.V, "W": fields.W}
    t0 = time.perf_counter()
    out = api.advection_step(arrays, DX, DY, DZ, HALO, fields.scalars)
    first = time.perf_counter() - t0
    # each step is a bounded sample: whole steps while the run fits in about two minutes, else a z-slab
    budget_s = 120.0
    nz_sample = NZ
    if first * (warmup + args.steps) > budget_s:
        nz_sample = max(8, int(NZ * budget_s / (first * (warmup + args.steps))))
        geo = wl.Geometry(NX, NY, nz_sample, halo=HALO, dx=DX, dy=DY, dz=DZ)
        fields = wl.advection_fields(geo, seed=0, nscalar=NSCALAR)
        arrays = {"U": fields.U, "V": fields.V, "W": fields.W}
        out = api.advection_step(arrays, DX, DY, DZ, HALO, fields.scalars)
    for _ in range(warmup - 1):
        api.advection_step(arrays, DX, DY, DZ, HALO, fields.scalars, out=out)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        api.advection_step(arrays, DX, DY, DZ, HALO, fields.scalars, out=out)
    elapsed = time.perf_counter() - t0
    value = geo.points * args.steps / elapsed / 1e9
    cores = api.threads()
    sample = (f"{args.steps} steps of {NX}x{NY}x{nz_sample} (U,V,W + 3 scalars)"
              + ("" if nz_sample == NZ else f"; z-slab of the {NZ}-level workload"))
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": warmup, "ms_per_step": elapsed / args.steps * 1e3 * NZ / nz_sample, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded sine modes + noise)",
        "config": {"workload": "advection 512x512x128 halo 2 + 3 scalars, tendency step", "nx": NX, "ny": NY,
                   "nz": NZ, "halo": HALO, "scalars": NSCALAR},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                         "note": "C restatement of cdu.f90/cvd.f90/cdw.f90 (-O3 -fopenmp -ffp-contract=off); "
                                 "the reference's Fortran control needs gfortran, absent on both machines"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    parser = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=50)
    parser.add_argument("--warmup", type=int, default=3)
    parser.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    parser.add_argument("--no-cpu-baseline", action="store_true")
    parser.add_argument("--size", type=int, nargs=3, metavar=("NX", "NY", "NZ"),
                        help="override the grid (profiling captures of a smaller case)")
    args = parser.parse_args()
    args.warmup = max(3, args.warmup)
    if args.size:
        global NX, NY, NZ
        NX, NY, NZ = args.size
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
