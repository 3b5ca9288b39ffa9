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
import gc
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


def fp64_ops_per_point(nscalar: int, numerics: str = "strict", mode: str = "tendency") -> int:
    """FP64-pipe instructions per point of each kernel's expression DAG (every face value computed once).

    Products on the integer pipes (``mul_rn_int``, rounded exactly as DMUL) and the exact halving (an exponent
    decrement) are not counted here (``int_pipe_ops_per_point``).
    strict (the reference grouping): U, V, W: 9 face sums, 15 flux differences, 30 advective-form sums and
    differences, and the first product of each of the 9 face fluxes (the second product of each flux and the 18
    advective-form products run on the integer pipes); scalars: 3 shared coefficient products, and per scalar 8
    sums and differences and 3 face-flux products.
    fast (factored FMA form): U, V, W: 6 face sums + 12 per component (3 for the direction along it, 3 for each
    across, 3 to accumulate, of which a tendency's first is a plain product); scalars: 5 for the shared divergence
    term + 7 FMAs per scalar (6 in a tendency).
    """
    tendency = mode == "tendency"
    if numerics == "fast":
        return 6 + 3 * (12 - tendency) + (5 + (7 - tendency) * nscalar if nscalar else 0)
    return 63 + (3 + 11 * nscalar if nscalar else 0)


def int_pipe_ops_per_point(nscalar: int, numerics: str = "strict", mode: str = "tendency") -> int:
    """Floating-point operations per point that run on the integer pipes: products, and the strict kernel's exact
    halving of U, V, W."""
    tendency = mode == "tendency"
    if numerics == "fast":
        return 9 + 3 * tendency + (3 + tendency * nscalar if nscalar else 0)
    return 27 + 3


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

    summary_cache = None

    def summary(self):
        if self.summary_cache is not None:
            return self.summary_cache
        self.summary_cache = self._summary()
        return self.summary_cache

    def _summary(self):
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
    """One process per GPU under torchrun: (dist or None, rank, world, local rank). NCCL with GPUs, gloo without."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        dist.init_process_group(backend="nccl" if torch.cuda.is_available() else "gloo")
        return dist, rank, world, local
    return None, rank, world, local


def barrier(dist, torch):
    if dist is None:
        return
    if dist.get_backend() == "nccl":
        dist.barrier(device_ids=[torch.cuda.current_device()])
    else:
        dist.barrier()


def max_over_ranks(dist, torch, value: float) -> float:
    if dist is None:
        return value
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(points_per_rank: int, world: int, steps: int, slowest_ms: float) -> float:
    """Gpts/s of the whole job: every rank's points x steps over the slowest rank's time (replicas, weak scaling)."""
    return points_per_rank * world * steps / (slowest_ms * 1e-3) / 1e9


def cpu_model() -> str:
    """The host CPU's model name (lscpu), for the CPU baseline's record."""
    try:
        text = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
    except (OSError, subprocess.SubprocessError):
        return "unknown"
    for line in text.splitlines():
        if line.startswith("Model name:"):
            return line.split(":", 1)[1].strip()
    return "unknown"


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
    return geo.points / t / 1e9, api.threads(), f"{len(times)} full steps (median) after 1 warm-up", out


def parity_report(device_outputs, oracle_out, geo, names):
    """Per field: normwise max relative error, pointwise max relative error (1e-300 floor, over points
    above 1e-3 of the field's maximum) and the fraction of bit-identical interior values, against the oracle."""
    inner = geo.interior()
    report = {}
    for name, dev in zip(names, device_outputs):
        got = dev[inner]
        ref = oracle_out[name][inner]
        d = np.abs(got - ref)
        scale = float(np.abs(ref).max())
        big = np.abs(ref) >= 1e-3 * scale
        report[name] = {
            "normwise_rel": float(d.max() / scale) if scale else float(d.max()),
            "pointwise_rel": float((d[big] / np.maximum(np.abs(ref[big]), 1e-300)).max()) if big.any() else 0.0,
            "bit_identical": int(np.count_nonzero(got.view(np.int64) == ref.view(np.int64))),
            "bit_identical_frac": float(np.count_nonzero(got.view(np.int64) == ref.view(np.int64)) / got.size),
        }
    return report


def run_e2e(fields, steps, warmup, dist, torch, fast_fp=False):
    """Gpts/s of the step through the residency runtime and the generated entry, host buffers in and out.

    The warm-up takes the runtime through its one-time work: the first step runs the plain path, the first
    slab step launches directly and the second instantiates its graph, which later steps replay."""
    from compiler import emission, native
    import ctypes as c

    from compiler.resident.domain import ResidentDomain
    from compiler.runtime import abi

    geo = fields.geometry
    lib = native.runtime()
    functions = emission.bind(lib)
    dom = ResidentDomain(lib, fast_fp=fast_fp)
    inputs = fields.arrays()
    outputs = [np.zeros_like(a) for a in inputs]
    dom.begin_epoch()
    h_in = [dom.bind_real64(a) for a in inputs]
    h_out = [dom.bind_real64(a) for a in outputs]
    arrays = [*h_out[:3], *h_in[:3], *h_in[3:], *h_out[3:]]
    grid = [geo.nx, geo.ny, geo.nz, geo.halo]
    entry = f"advection::step{len(inputs) - 3}"

    phases, device = [], []
    timing = abi.SlabTiming()

    def step():
        t0 = time.perf_counter()
        dom.host_modify(h_in)
        t1 = time.perf_counter()
        status = emission.call(functions, entry, dom.context, abi.GPU, arrays, [geo.dx, geo.dy, geo.dz], grid)
        if status != abi.OK:
            raise RuntimeError(f"{entry} returned {status}: {lib.fort_scope_error().decode()}")
        t2 = time.perf_counter()
        dom.observe(h_out)
        t3 = time.perf_counter()
        phases.append(((t1 - t0) * 1e3, (t2 - t1) * 1e3, (t3 - t2) * 1e3))
        # the device timeline of the step's slab pipeline (recorded by the runtime; the step is complete)
        device.append(timing.as_dict() if lib.fort_scope_slab_timing_get_v1(dom.context, c.byref(timing)) == abi.OK
                      else None)

    for k in range(max(3, warmup)):
        step()
        if k == 0:
            dom.require(lib.fort_scope_slab_timing_set_v1(dom.context, 1))
    phases.clear()
    device.clear()
    n = max(1, min(steps, 40))
    gc_was = gc.isenabled()
    gc.disable()  # the timed steps allocate little; a collection inside one would be the interpreter's, not ours
    barrier(dist, torch)
    t0 = time.perf_counter()
    marks = [t0]
    for _ in range(n):
        step()
        marks.append(time.perf_counter())
    elapsed = marks[-1] - t0
    if gc_was:
        gc.enable()
    steps_ms = [(b - a) * 1e3 for a, b in zip(marks, marks[1:])]
    per_step = sorted(steps_ms)
    elapsed = max_over_ranks(dist, torch, elapsed)
    dom.end_epoch()
    dom.close()
    world = dist.get_world_size() if dist is not None else 1
    nbytes = sum(a.nbytes for a in inputs)
    median = per_step[len(per_step) // 2]
    slowest = max(range(n), key=lambda k: steps_ms[k])
    spread = {"min": per_step[0], "median": median, "max": per_step[-1],
              "slowest_step": {"index": slowest, "ms": steps_ms[slowest],
                               "host_modify_ms": phases[slowest][0], "entry_call_ms": phases[slowest][1],
                               "observe_ms": phases[slowest][2], "device": device[slowest]},
              "median_device": ({k: statistics.median(d[k] for d in device) for k in device[0]}
                                if all(device) else None),
              "median_phases_ms": {name: statistics.median(ph[k] for ph in phases)
                                   for k, name in enumerate(("host_modify", "entry_call", "observe"))},
              "steps_over_1.5x_median": sum(1 for t in steps_ms if t > 1.5 * median)}
    return geo.points * world * n / elapsed / 1e9, n, nbytes, outputs, spread


KERNELS = {"fast": 2, "strict": 0}  # enum f2c_kernel_variant: F2C_KERNEL_FAST, F2C_KERNEL_FACES


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
    outs = {name: [torch.zeros_like(t) for t in dev_in] for name in KERNELS}
    grid = native.make_grid(NX, NY, NZ, HALO, DX, DY, DZ)
    p = [t.data_ptr() for t in dev_in]
    stream = torch.cuda.Stream()
    primary = args.numerics
    secondary = "strict" if primary == "fast" else "fast"

    def launcher(name):
        q = [t.data_ptr() for t in outs[name]]
        variant = KERNELS[name]
        return lambda s: native.advection(grid, *p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:], stream=s,
                                          variant=variant)

    def captured(fn):
        with torch.cuda.stream(stream):
            fn(stream.cuda_stream)  # warm the module before capture
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            fn(stream.cuda_stream)
        return graph

    def timed(graph, steps):
        for _ in range(args.warmup):
            graph.replay()
        torch.cuda.synchronize()
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        barrier(dist, torch)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            start.record(stream)
            for _ in range(steps):
                graph.replay()
            stop.record(stream)
        torch.cuda.synchronize()
        barrier(dist, torch)
        return max_over_ranks(dist, torch, start.elapsed_time(stop))

    # the headline: one step (one launch) captured as a CUDA graph and replayed
    graph = captured(launcher(primary))
    with ClockSampler(local) as sampler:
        elapsed_ms = timed(graph, args.steps)
    ms_per_step = elapsed_ms / args.steps
    points = geo.points
    value = whole_job_value(points, world, args.steps, elapsed_ms)
    # the other numerical contract's kernel on the same inputs
    other_steps = max(3, min(args.steps, 20))
    other_ms = timed(captured(launcher(secondary)), other_steps) / other_steps

    # The reference's emitted structure on the same GPU: per momentum component the set, flux-form,
    # advective-form and halving procedures as separate grid-stride launches, the scalars as one more launch.
    u_, v_, w_ = p[:3]
    q_ref = [t.data_ptr() for t in outs["strict"]]

    def reference_structure(s):
        ops = ((native.CDU_DIV, native.CDU_ADV), (native.CDV_DIV, native.CDV_ADV), (native.CDW_DIV, native.CDW_ADV))
        for o, (div, adv) in zip(q_ref[:3], ops):
            native.procedure(native.SET, grid, o, value=0.0, stream=s)
            native.procedure(div, grid, o, u_, v_, w_, stream=s)
            native.procedure(adv, grid, o, u_, v_, w_, stream=s)
            native.procedure(native.MULTIPLY, grid, o, value=0.5, stream=s)
        native.advection(grid, u_, v_, w_, scalars=p[3:], scalar_out=q_ref[3:], stream=s)

    reference_ms = _graph_time(torch, stream, reference_structure, max(3, min(args.steps, 20)), args.warmup)
    # the strict kernel's outputs again (the structure above wrote the same values; recompute for clarity)
    launcher("strict")(stream.cuda_stream)
    torch.cuda.synchronize()

    # FP64 pipe rate of this GPU (the roofline that binds first on GB300), from the bench's own probe library
    scratch = torch.empty(8 * torch.cuda.get_device_properties(local).multi_processor_count * 256,
                          dtype=torch.float64, device="cuda")
    fp64_add = native.fp64_rate(0, scratch.data_ptr(), scratch.numel())
    fp64_fma = native.fp64_rate(1, scratch.data_ptr(), scratch.numel())
    del scratch

    # End to end through the reference-facing C ABI: a residency domain (in the headline's numerical contract)
    # holds the host arrays (pinned in place at registration), every step the host rewrites the inputs (their
    # device copies go stale), the generated entry advection::step3 runs (uploading what changed) and the
    # outputs are published back.
    e2e_value, e2e_steps, bytes_in, e2e_outputs, e2e_spread = run_e2e(fields, args.steps, args.warmup, dist, torch,
                                                                      fast_fp=primary == "fast")
    bytes_out = sum(a.nbytes for a in e2e_outputs)
    # the host arrays the end-to-end path published equal, bit for bit, what the graph-replayed launches of the
    # same kernel left on the device from the same inputs: the end-to-end steps did the whole step
    e2e_matches = all(np.array_equal(a.view(np.int64), t.cpu().numpy().view(np.int64))
                      for a, t in zip(e2e_outputs, outs[primary]))
    del e2e_outputs

    peak, peak_kind = hbm_peak()
    alg = algorithmic_bytes_per_point(NSCALAR) * points
    achieved = alg / (ms_per_step * 1e-3) / 1e9
    traffic = None
    traffic_file = ROOT / "profiles" / f"advection_{primary}_512x512x128_s3_traffic.txt"
    if traffic_file.exists():
        for line in traffic_file.read_text().splitlines():
            if line.startswith("dram_bytes_per_launch"):
                traffic = float(line.split("=")[1])
    fp64_peak = max(fp64_add, fp64_fma)

    clock_mhz = sampler.summary().get("sm_mhz") or 2070.0
    nominal_fp64 = 2.0 * torch.cuda.get_device_properties(local).multi_processor_count * clock_mhz * 1e6

    def fp64_roofline(name, ms):
        ops = fp64_ops_per_point(NSCALAR, name)
        rate = ops * points / (ms * 1e-3)
        return {"achieved_ops_per_s": rate, "peak_ops_per_s": fp64_peak, "frac": rate / fp64_peak,
                "ops_per_point": ops, "int_pipe_ops_per_point": int_pipe_ops_per_point(NSCALAR, name)}

    kernel_ms = {primary: ms_per_step, secondary: other_ms}
    kernel_names = {"fast": "advection_fast_kernel<3,7,8,3>", "strict": "advection_faces_kernel<3,7>"}
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded sine modes + noise, scalars)",
        "config": config_object(world),
        "numerics": {"fast": "fast-fp (the reference's --fast-fp contract): FMA contraction and factored sums, every "
                             "field within 1e-12 of its maximum of the strict result (see parity)",
                     "strict": "strict (bit-identical to the oracle)"}[primary],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": f"{peak_kind} hbm_gbs",
                     "algorithmic_bytes_per_launch": alg, "kernel": kernel_names[primary]},
        "fp64_roofline": {**fp64_roofline(primary, ms_per_step), "peak_add_rn": fp64_add, "peak_fma_rn": fp64_fma,
                          "peak_source": "measured live", "kernel": kernel_names[primary],
                          # the instruction rate ncu states for the FP64 pipe: 2 lanes per clock per SM
                          "nominal_ops_per_s": nominal_fp64,
                          "frac_of_nominal": fp64_roofline(primary, ms_per_step)["achieved_ops_per_s"] / nominal_fp64},
        secondary if secondary == "strict" else "fast_fp": {
            "value": whole_job_value(points, world, 1, other_ms), "ms_per_step": other_ms, "steps": other_steps,
            "kernel": kernel_names[secondary], "fp64_roofline": fp64_roofline(secondary, other_ms)},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": bytes_in,
                "d2h_bytes_per_step": bytes_out, "steps": e2e_steps, "step_ms": e2e_spread,
                "outputs_equal_device_path": e2e_matches, "numerics": primary,
                "path": "fort_scope runtime + generated entry advection::step3; the host rewrites the inputs and reads "
                        "the outputs every step, so from the second round the step runs as z-slabs whose uploads "
                        "(copy stream), kernels and publications (second copy stream) overlap; host arrays pinned "
                        "in place, copies by DMA over NVLink-C2C"},
        "gpu_launches": args.steps,
        "clocks": sampler.summary(),
        "reference_structure": {"value": whole_job_value(points, world, 1, reference_ms), "ms_per_step": reference_ms,
                                "how": "the reference's emitted structure on this GPU: set, flux form, advective form "
                                       "and halving as separate launches per momentum component, plus one launch "
                                       "for the scalars; graph-replayed"},
    }
    if primary == "fast":
        result["fast_fp"] = {"value": value, "ms_per_step": ms_per_step, "steps": args.steps,
                             "kernel": kernel_names["fast"], "headline": True}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, sample, oracle_out = cpu_oracle_sample(fields)
        result["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                                  "cpu": cpu_model(), "nproc": os.cpu_count()}
        names = ["U", "V", "W", *[f"S{n}" for n in range(NSCALAR)]]
        parity = {}
        for name in KERNELS:
            parity[name] = parity_report([t.cpu().numpy() for t in outs[name]], oracle_out, geo, names)
        result["parity"] = {"against": "the C oracle on the same inputs (full 512x512x128 step)", **parity,
                            "max_normwise_rel": {k: max(f["normwise_rel"] for f in v.values())
                                                 for k, v in parity.items()}}
        result["fast_fp"]["max_normwise_rel"] = result["parity"]["max_normwise_rel"]["fast"]
        del oracle_out
    if rank == 0 and world == 1 and not args.no_batched:
        result["batched"] = batched_summary(args, torch)
    if rank == 0 and world == 1 and not args.no_serving:
        result["serving"] = serving_summary(args, torch)
    if rank == 0:
        print(json.dumps(result), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def config_object(world: int = 1) -> dict:
    """The workload's config, identical in both arms."""
    return {"workload": "advection 512x512x128 halo 2 + 3 scalars, tendency step, CUDA graph replay",
            "nx": NX, "ny": NY, "nz": NZ, "halo": HALO, "scalars": NSCALAR,
            "parallelism": f"replicas x{world}", "l2": "inputs 3.4 GB > L2, no flush"}


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
        "config": config_object(1),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                         "cpu": cpu_model(), "nproc": os.cpu_count(),
                         "note": "C restatement of cdu.f90/cvd.f90/cdw.f90 (-O3 -fopenmp -ffp-contract=off); "
                                 "the reference's Fortran control needs gfortran, absent on both machines"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def _graph_time(torch, stream, fn, steps, warmup):
    """Milliseconds per replay of a CUDA graph that captures ``fn(stream)``, timed with events on ``stream``."""
    with torch.cuda.stream(stream):
        fn(stream.cuda_stream)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        fn(stream.cuda_stream)
    for _ in range(warmup):
        graph.replay()
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        start.record(stream)
        for _ in range(steps):
            graph.replay()
        stop.record(stream)
    torch.cuda.synchronize()
    return start.elapsed_time(stop) / steps


def _stream_time(torch, stream, fn, steps, warmup):
    """ms per call of ``fn(stream)`` (which launches its own graph), CUDA events on the stream."""
    for _ in range(warmup):
        fn(stream.cuda_stream)
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        fn(stream.cuda_stream)
    stop.record(stream)
    torch.cuda.synchronize()
    return start.elapsed_time(stop) / steps


def ensemble_measure(torch, count, steps, warmup, tune=False, numerics=("fast", "strict")):
    """The ensemble configuration: ``count`` uneven instances (nx, ny from {64..256}, nz from {32, 64, 96}, seed 1),
    U, V, W + 1 scalar. Per numerical contract: one persistent launch per step (autotuned z-chunks) against the
    same instances one plain launch at a time, both graph-replayed on the same stream."""
    from compiler import native, scheduling
    from compiler import workloads as wl

    shapes = wl.ensemble_shapes(64, seed=1)[:count]
    nscalar = 1
    inst = []
    for n, (nx, ny, nz) in enumerate(shapes):
        geo = wl.Geometry(nx, ny, nz, halo=HALO, dx=DX, dy=DY, dz=DZ)
        ins = wl.advection_fields_device(geo, 1000 + n, nscalar, torch)
        outs = [torch.empty_like(t) for t in ins]
        p, q = [t.data_ptr() for t in ins], [t.data_ptr() for t in outs]
        grid = native.make_grid(nx, ny, nz, HALO, DX, DY, DZ)
        inst.append((geo, ins, outs, grid, native.make_fields(*p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:])))
    points = sum(x[0].points for x in inst)
    stream = torch.cuda.Stream()
    gpu = torch.cuda.get_device_name(0)

    def batch_time(kz, fast, rows=8, n_steps=5, n_warmup=3):
        # one step = one replay of the batch's own CUDA graph (counter reset + persistent launch)
        batch = native.Batch([x[3] for x in inst], [x[4] for x in inst], kz=kz, tile_rows=rows)
        ws = torch.empty(batch.workspace_bytes(), dtype=torch.uint8, device="cuda")
        batch.prepare(ws.data_ptr(), ws.numel(), stream.cuda_stream)
        batch.set_fast_fp(fast)
        return _stream_time(torch, stream, lambda s: batch.graph_step(s), n_steps, n_warmup) * 1e-3

    def resident_entries_time(fast, n_steps, n_warmup):
        # each instance alone, one after another, through the residency runtime: its steps are calls of the
        # generated entry advection::step<N> inside one epoch, with its fields already resident on the device
        from compiler import emission
        from compiler.resident.domain import ResidentDomain
        from compiler.runtime import abi

        lib = native.runtime()
        functions = emission.bind(lib)
        dom = ResidentDomain(lib, fast_fp=fast)
        dom.begin_epoch()
        calls = []
        try:
            for geo, ins, outs, grid, fields in inst:
                h_in = [dom.bind_real64(t.cpu().numpy()) for t in ins]
                h_out = [dom.bind_real64(np.zeros(tuple(t.shape))) for t in outs]
                calls.append((f"advection::step{len(ins) - 3}", [*h_out[:3], *h_in[:3], *h_in[3:], *h_out[3:]],
                              [geo.dx, geo.dy, geo.dz], [geo.nx, geo.ny, geo.nz, geo.halo]))

            def run(count):
                for entry, arrays, reals, ints in calls:
                    for _ in range(count):
                        status = emission.call(functions, entry, dom.context, abi.GPU, arrays, reals, ints)
                        if status != abi.OK:
                            raise RuntimeError(f"{entry} returned {status}: {lib.fort_scope_error().decode()}")

            run(max(1, n_warmup))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            run(n_steps)
            torch.cuda.synchronize()
            return (time.perf_counter() - t0) / n_steps
        finally:
            dom.end_epoch()
            dom.close()

    tuned = {}
    if tune:
        for name in numerics:
            tuned[name] = scheduling.tune(shapes, gpu, nscalar, lambda kz, rows: batch_time(kz, name == "fast", rows),
                                          numerics=name)
    out = {"instances": len(shapes), "points": points, "steps": steps, "warmup": warmup, "tuned": tuned or None}
    with ClockSampler(0) as sampler:
        for name in numerics:
            fast = name == "fast"
            kz = scheduling.kz_for(shapes, gpu, nscalar, numerics=name)
            rows = scheduling.rows_for(gpu, nscalar, numerics=name)
            batched_s = batch_time(kz, fast, rows, n_steps=steps, n_warmup=warmup)
            variant = native.FAST if fast else native.FACES

            def one_at_a_time(s):
                for geo, ins, outs, grid, fields in inst:
                    p, q = [t.data_ptr() for t in ins], [t.data_ptr() for t in outs]
                    native.advection(grid, *p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:], stream=s,
                                     variant=variant)

            plain_ms = _graph_time(torch, stream, one_at_a_time, steps, warmup)
            entries_s = resident_entries_time(fast, steps, warmup)
            value, plain = points / batched_s / 1e9, points / (plain_ms * 1e-3) / 1e9
            entries = points / entries_s / 1e9
            out[name] = {"value": value, "ms_per_step": batched_s * 1e3,
                         "shapes": {"tile": f"32x{rows}",
                                    "kz": {scheduling.bucket(nz): k for (_, _, nz), k in zip(shapes, kz)}},
                         "plain_resident": {"value": plain, "ms_per_step": plain_ms,
                                            "how": f"{len(shapes)} single-instance launches per step, one graph"},
                         "batched_over_plain": value / plain,
                         "resident_entries": {"value": entries, "ms_per_step": entries_s * 1e3,
                                              "how": "each instance alone, one after another, its steps through the "
                                                     "generated entry advection::step1 in a residency epoch, fields "
                                                     "resident; wall clock with a device synchronisation either side"},
                         "batched_over_resident_entries": value / entries}
    out["clocks"] = sampler.summary()
    return out, inst, stream


def batched_summary(args, torch):
    """The compact ensemble object of the default bench line (64 instances, at least 20 steps)."""
    steps = max(20, min(args.steps, 50))
    out, inst, _ = ensemble_measure(torch, 64, steps, args.warmup)
    del inst
    torch.cuda.empty_cache()
    return out


def serving_summary(args, torch):
    """The compact serving object of the default bench line: two arrival rates, 500 jobs each."""
    from compiler import serving

    count = max(20, args.jobs)
    serving.warm_up(torch, args.numerics)
    rates = []
    with ClockSampler(0) as sampler:
        for rate in (200.0, 2000.0):
            r = serving.measure_rate(torch, rate, count, args.numerics)
            cb, serial, model = r["continuous_batching"], r["serial_plain"], r["serial_device_model"]
            rates.append({"rate_jobs_per_s": rate, "jobs": count,
                          "continuous_batching": {k: cb[k] for k in ("gpts_per_s", "jobs_per_s", "p50_ms", "p99_ms",
                                                                     "wall_s", "ticks")},
                          "server": {k: cb["server"][k] for k in ("graph_builds", "graph_replays", "plan_builds",
                                                                  "bursts", "peak_active", "peak_job_bytes",
                                                                  "refused_admissions")},
                          "serial_plain": {k: serial[k] for k in ("gpts_per_s", "p50_ms", "p99_ms", "wall_s")},
                          "serial_device_model": {k: model[k] for k in ("gpts_per_s", "p50_ms", "p99_ms")},
                          "throughput_ratio": r["throughput_ratio"], "over_device_model": r["over_device_model"]})
    return {"numerics": args.numerics, "config": serving.config(), "rates": rates, "clocks": sampler.summary()}


def run_batched(args):
    """64 uneven instances (nx, ny from {64..256}, nz from {32, 64, 96}, seed 1), U, V, W + 1 scalar.

    ``--instances N`` takes the first N of the same draw (profiling captures of a smaller case)."""
    import torch

    from compiler import native

    torch.cuda.set_device(0)
    out, inst, stream = ensemble_measure(torch, args.instances, args.steps, args.warmup, tune=args.tune)
    points = out["points"]

    def per_procedure(s):
        # the reference resident build's structure: set, div, adv, multiply per component, one instance
        # at a time, and the scalar as its own launch
        ops = ((native.CDU_DIV, native.CDU_ADV), (native.CDV_DIV, native.CDV_ADV), (native.CDW_DIV, native.CDW_ADV))
        for geo, ins, outs, grid, fields in inst:
            u, v, w = (t.data_ptr() for t in ins[:3])
            for o_, (div, adv) in zip(outs[:3], ops):
                o = o_.data_ptr()
                native.procedure(native.SET, grid, o, value=0.0, stream=s)
                native.procedure(div, grid, o, u, v, w, stream=s)
                native.procedure(adv, grid, o, u, v, w, stream=s)
                native.procedure(native.MULTIPLY, grid, o, value=0.5, stream=s)
            native.advection(grid, u, v, w, scalars=[ins[3].data_ptr()], scalar_out=[outs[3].data_ptr()],
                             stream=s)

    procedure_ms = _graph_time(torch, stream, per_procedure, max(3, args.steps // 4), args.warmup)
    procedure_rate = points / (procedure_ms * 1e-3) / 1e9
    head = out[args.numerics]
    print(json.dumps({
        "metric": f"batched ensemble Gpts/s ({out['instances']} uneven instances, U,V,W + 1 scalar, one persistent "
                  "launch per step)",
        "value": head["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": head["ms_per_step"], "higher_is_better": True, "dtype": "f64", "data": "synthetic (seeded)",
        "numerics": args.numerics,
        "config": {"workload": f"{out['instances']} instances, nx,ny in {{64..256}}, nz in {{32,64,96}}, seed 1",
                   "points": points, "shapes": head["shapes"]},
        "plain_resident": head["plain_resident"], "batched_over_plain": head["batched_over_plain"],
        "resident_entries": head["resident_entries"],
        "batched_over_resident_entries": head["batched_over_resident_entries"],
        "per_numerics": {k: out[k] for k in ("fast", "strict")},
        "reference_style_resident": {"value": procedure_rate, "ms_per_step": procedure_ms,
                                     "how": "per instance: set, div, adv, multiply for U, V, W + 1 scalar launch "
                                            f"(13 launches), {out['instances']} instances one at a time, one graph"},
        "batched_over_reference_style": head["value"] / procedure_rate,
        "tuned": out["tuned"], "gpu_launches": args.steps, "clocks": out["clocks"]}), flush=True)


def run_small(args):
    """The 64 x 64 x 32 configuration: 10 forward-Euler steps at dt = 0.1 with the boundary fill, as one graph."""
    import torch

    from compiler import native
    from compiler import workloads as wl

    geo = wl.Geometry(64, 64, 32, halo=HALO, dx=DX, dy=DY, dz=DZ)
    f = wl.advection_fields(geo, seed=0, nscalar=0)
    a = [torch.from_numpy(x).cuda() for x in f.arrays()]
    b = [torch.zeros_like(x) for x in a]
    grid = native.make_grid(geo.nx, geo.ny, geo.nz, geo.halo, geo.dx, geo.dy, geo.dz)

    def ten_steps(variant):
        def launch(s):
            src, dst = a, b
            for _ in range(10):
                native.advection(grid, *[t.data_ptr() for t in src], *[t.data_ptr() for t in dst],
                                 mode=native.ADVANCE_FILLED, dt=0.1, stream=s, variant=variant)
                src, dst = dst, src
        return launch

    stream = torch.cuda.Stream()
    us = {name: _graph_time(torch, stream, ten_steps(KERNELS[name]), args.steps, args.warmup) * 1e3 / 10
          for name in (args.numerics, "strict" if args.numerics == "fast" else "fast")}
    head = us[args.numerics]
    print(json.dumps({
        "metric": "64x64x32 advance step latency (U,V,W Euler dt=0.1 + boundary fill; 10 steps per graph)",
        "value": head, "unit": "us/step", "higher_is_better": False, "gpts_per_s": geo.points / head / 1e3,
        "numerics": args.numerics, "us_per_step": us,
        "steps": args.steps * 10, "warmup": args.warmup, "dtype": "f64", "data": "synthetic (seeded sine modes)",
        "config": {"workload": "64x64x32 halo 2, one launch per step (advance and boundary fill)",
                   "l2": "resident in L2: latency, not roofline"},
        "gpu_launches": args.steps * 10}), flush=True)


def run_stencils(args):
    """Diffusion 7-point on 384^3, Jacobi 5-point on 8192^2, Yee on 4096^2; uniform[0,1) inputs, zero boundaries."""
    import ctypes

    import torch

    from compiler import native

    lib = native.load()
    lib.f2c_diffusion7_v1.argtypes = [ctypes.POINTER(native.Grid), ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
    lib.f2c_jacobi5_v1.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_int64] * 4 + [ctypes.c_void_p]
    lib.f2c_yee2d_v1.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int64] * 4 + [ctypes.c_double] * 2 + [ctypes.c_void_p]
    peak, _ = hbm_peak()
    g = torch.Generator(device="cuda").manual_seed(0)
    stream = torch.cuda.Stream()
    results = {}

    def field(shape):
        t = torch.zeros(shape, dtype=torch.float64, device="cuda")
        inner = t[(slice(1, -1),) * len(shape)]
        inner.copy_(torch.rand(inner.shape, generator=g, device="cuda", dtype=torch.float64))
        return t

    n = 384
    a, b = field((n + 2,) * 3), torch.zeros((n + 2,) * 3, dtype=torch.float64, device="cuda")
    grid = native.make_grid(n, n, n, 1, 1.0, 1.0, 1.0)

    def diffuse(s):
        native.check(lib.f2c_diffusion7_v1(ctypes.byref(grid), a.data_ptr(), b.data_ptr(), 0.125, 1.0, s))
        native.check(lib.f2c_diffusion7_v1(ctypes.byref(grid), b.data_ptr(), a.data_ptr(), 0.125, 1.0, s))

    ms = _graph_time(torch, stream, diffuse, args.steps, args.warmup) / 2
    results["diffusion7_384^3"] = {"ms_per_step": ms, "gpts_per_s": n ** 3 / ms / 1e6,
                                   "hbm_frac": 16 * n ** 3 / (ms * 1e-3) / 1e9 / peak, "fp64_ops_per_point": 7,
                                   "int_pipe_ops_per_point": 3}
    del a, b
    n = 8192
    u, v = field((n + 2, n + 2)), torch.zeros((n + 2, n + 2), dtype=torch.float64, device="cuda")

    def sweep(s):
        native.check(lib.f2c_jacobi5_v1(u.data_ptr(), v.data_ptr(), n, n, 1, n + 2, s))
        native.check(lib.f2c_jacobi5_v1(v.data_ptr(), u.data_ptr(), n, n, 1, n + 2, s))

    ms = _graph_time(torch, stream, sweep, args.steps, args.warmup) / 2
    results["jacobi5_8192^2"] = {"ms_per_step": ms, "gpts_per_s": n * n / ms / 1e6,
                                 "hbm_frac": 16 * n * n / (ms * 1e-3) / 1e9 / peak, "fp64_ops_per_point": 3,
                                 "int_pipe_ops_per_point": 1}
    del u, v
    n = 4096
    ez, hx, hy = (field((n + 2, n + 2)) for _ in range(3))

    def leap(s):
        native.check(lib.f2c_yee2d_v1(ez.data_ptr(), hx.data_ptr(), hy.data_ptr(), n, n, 1, n + 2, 0.5, 0.7, s))

    ms = _graph_time(torch, stream, leap, args.steps, args.warmup)
    results["yee2d_4096^2"] = {"ms_per_step": ms, "gpts_per_s": n * n / ms / 1e6,
                               "hbm_frac": 48 * n * n / (ms * 1e-3) / 1e9 / peak, "fp64_ops_per_point": 8,
                               "int_pipe_ops_per_point": 3}
    print(json.dumps({"metric": "generality stencils Gpts/s (100-step graphs)", "unit": UNIT, "dtype": "f64",
                      "steps": args.steps, "warmup": args.warmup, "results": results,
                      "peak_hbm_gbs": peak}), flush=True)


def main():
    parser = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=200)
    parser.add_argument("--warmup", type=int, default=3)
    parser.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    parser.add_argument("--no-cpu-baseline", action="store_true")
    parser.add_argument("--no-batched", action="store_true", help="leave the ensemble object out of the line")
    parser.add_argument("--no-serving", action="store_true", help="leave the serving object out of the line")
    parser.add_argument("--numerics", choices=("fast", "strict"), default="fast",
                        help="the headline kernel: fast-fp (default; within 1e-12 of the oracle) or strict "
                             "(bit-identical); the other is timed beside it")
    parser.add_argument("--size", type=int, nargs=3, metavar=("NX", "NY", "NZ"),
                        help="override the grid (profiling captures of a smaller case)")
    parser.add_argument("--workload", choices=("advection", "batched", "small", "stencils", "serving"),
                        default="advection", help="the headline step (default) or another configuration")
    parser.add_argument("--tune", action="store_true", help="batched: run the z-chunk autotuner first")
    parser.add_argument("--instances", type=int, default=64, help="batched: the first N instances of the ensemble")
    parser.add_argument("--jobs", type=int, default=500, help="serving: jobs per arrival rate")
    parser.add_argument("--rates", type=float, nargs="+", help="serving: arrival rates (jobs/s) of --workload serving")
    args = parser.parse_args()
    args.warmup = max(3, args.warmup)
    if args.size:
        global NX, NY, NZ
        NX, NY, NZ = args.size
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "small":
        run_small(args)
    elif args.workload == "stencils":
        run_stencils(args)
    elif args.workload == "serving":
        from compiler.serving import bench_main

        bench_main(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
