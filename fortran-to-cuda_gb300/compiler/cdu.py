"""The cdu benchmark driver, run as the resident build runs it.

``python -m compiler.cdu [--nx 64 --ny 64 --nz 64 --iterations 100 --warmup 5 --seed 20261123] [--fast-fp]``

Restates ``benchmarks/cdu/src/main.f90`` (allocation :47-51, dx = 1/N :54-56,
warm-up and timed loop :67-79, report :86-92) with the residency directives
``cdu.toml`` adds: the epoch opens before the warm-up (``!$fort enter``),
closes before the clock stops (``!$fort leave``, which publishes U2), and the
domain is closed before the arrays are freed (``!$fort close``). Each
``call CDU(...)`` is the generated entry of ``momentumadvection::cdu`` called
through the runtime exactly as the spliced call block calls it. The report has
the driver's lines and formats; the checksum is the sequential sum of the
interior of U2 in array-element order, as ``sum(real(U2(2:NX+1, ...), 8))``.

The fields are uniform [0, 1) from numpy's generator (gfortran's
``random_number`` cannot be reproduced here), one ghost layer, every value
drawn as ``random_number`` fills whole arrays. ``--fast-fp`` runs the driver
as a resident build prepared with the reference's ``--fast-fp`` runs it: the
domain's context under the fast-fp numerical contract.
"""

from __future__ import annotations

import argparse
import sys
import time

import numpy as np

from . import emission, native
from . import workloads as wl
from .resident.domain import ResidentDomain
from .runtime import abi


def sequential_sum(values: np.ndarray) -> float:
    """Left-to-right sum in array-element order (the order a sequential Fortran SUM takes)."""
    flat = np.ascontiguousarray(values).ravel()
    return float(np.cumsum(flat)[-1]) if flat.size else 0.0


def run(nx: int, ny: int, nz: int, iterations: int, warmup: int, seed: int, fast_fp: bool = False) -> dict:
    fields = wl.reference_driver_fields(nx, ny, nz, seed)
    geo = fields.geometry
    u, v, w = fields.U, fields.V, fields.W
    u2 = np.zeros_like(u)
    lib = native.runtime()
    entries = emission.bind(lib)
    dom = ResidentDomain(lib, fast_fp=fast_fp)
    reals, ints = [geo.dx, geo.dy, geo.dz], [nx, ny, nz]

    def cdu(handles):
        status = emission.call(entries, "momentumadvection::cdu", dom.context, abi.GPU, handles, reals, ints)
        if status != abi.OK:
            raise RuntimeError(f"CDU entry returned {status}: {lib.fort_scope_error().decode(errors='replace')}")

    dom.begin_epoch()                                   # !$fort enter
    handles = [dom.bind_real64(a) for a in (u2, u, v, w)]
    for _ in range(warmup):
        cdu(handles)
    start = time.perf_counter()
    for _ in range(iterations):
        cdu(handles)
    dom.end_epoch()                                     # !$fort leave: U2 is published
    total_ms = (time.perf_counter() - start) * 1e3
    dom.close()                                         # !$fort close
    interior = u2[1:nz + 1, 1:ny + 1, 1:nx + 1]
    return {"nx": nx, "ny": ny, "nz": nz, "iterations": iterations, "warmup": warmup, "total_ms": total_ms,
            "ms_per_iter": total_ms / iterations, "checksum": sequential_sum(interior), "u2": u2}


def report(r: dict) -> str:
    return "\n".join([
        "--- CDU benchmark ---",
        f"grid:         {r['nx']} x {r['ny']} x {r['nz']}",
        f"iterations:   {r['iterations']}",
        f"warmup_iters: {r['warmup']}",
        f"total_ms:     {r['total_ms']:14.3f} ms",
        f"ms_per_iter:  {r['ms_per_iter']:14.3f} ms",
        f"checksum:     {fortran_es(r['checksum'])}",
    ])


def fortran_es(x: float) -> str:
    """Fortran ES24.16: right-aligned in 24 columns, one digit before the point, 16 after, exponent E+dd."""
    mantissa, exponent = f"{x:.16E}".split("E")
    e = int(exponent)
    text = f"{mantissa}E{'+' if e >= 0 else '-'}{abs(e):02d}" if abs(e) < 100 else f"{mantissa}{'+' if e >= 0 else '-'}{abs(e):03d}"
    return text.rjust(24)


def main(argv=None) -> int:
    parser = argparse.ArgumentParser(prog="python -m compiler.cdu", description=__doc__.splitlines()[0])
    parser.add_argument("--nx", type=int, default=64)
    parser.add_argument("--ny", type=int, default=64)
    parser.add_argument("--nz", type=int, default=64)
    parser.add_argument("--iterations", type=int, default=100)
    parser.add_argument("--warmup", type=int, default=5)
    parser.add_argument("--seed", type=int, default=20261123)
    parser.add_argument("--fast-fp", action="store_true", help="the fast-fp numerical contract (FMA contraction)")
    args = parser.parse_args(argv)
    print(report(run(args.nx, args.ny, args.nz, args.iterations, args.warmup, args.seed, args.fast_fp)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
