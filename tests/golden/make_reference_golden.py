"""Writes tests/golden/reference_kernels.npz: golden vectors computed by the reference's own Fortran source.

The reference's procedures are executed from their source text as it lies in
the reference checkout (``F2C_REFERENCE_ROOT``, default the checkout this was
generated from) by the Fortran-subset interpreter ``fortran_kernels.py``
(IEEE binary64, the expression trees evaluated as written):

* ``benchmarks/cdu/src/cdu.f90`` (CDU, and each of set / CDUdiv / CDUadv /
  multiply), ``compiler/tests/fixtures/stencils/cvd.f90`` (CDV) and ``cdw.f90``
  (CDW), on uniform random U, V, W at three grids, with one ghost layer (the
  reference driver's layout) and with two (the arrays passed from the second
  layer, so the procedures see one);
* ``compiler/tests/apps/box/stepper.f90`` ``diffuse`` with its ``params``
  module (two ghost layers, lower bound -1 as declared there);
* the Jacobi sweep of ``compiler/tests/apps/relax/relax.f90`` (its DO nest,
  taken verbatim from the program and run on arrays of lower bound 0);
* the reference's own correctness-test programs for the three procedures,
  ``compiler/tests/fixtures/stencils/{cdu,cvd,cdw}_main.f90`` (deterministic
  sin/cos inputs, one call, the interior of the result written one value per
  line), at their default 16 x 16 x 16 and at 12 x 10 x 8 through their
  VAR_NX/VAR_NY/VAR_NZ macros: the written values and the inputs the programs
  built (sin and cos from this machine's C library) are stored.

Inputs are uniform in [0, 1) (velocities shifted to [-1, 1)), stored with the
outputs, so nothing of the platform's libm enters the check. Run from the
repository root: python tests/golden/make_reference_golden.py
"""

import os
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

from fortran_kernels import Source  # noqa: E402

REFERENCE = Path(os.environ.get("F2C_REFERENCE_ROOT", "/root/reference"))
OUT = HERE / "reference_kernels.npz"

# (nx, ny, nz, ghost layers, dx, dy, dz, seed)
ADVECTION_CASES = [(12, 10, 6, 1, 10.0, 10.0, 5.0, 11), (17, 9, 8, 2, 1.0 / 17, 0.3, 0.25, 12),
                   (16, 12, 8, 1, 0.125, 1.0 / 12, 0.7, 13)]
DIFFUSION_CASE = (16, 12, 10, 0.5, 0.01, 0.3, 21)   # nx, ny, nz, dx, dt, nu, seed
JACOBI_CASE = (48, 31)                              # n, seed


def advection_source() -> Source:
    return Source((REFERENCE / "benchmarks/cdu/src/cdu.f90").read_text(),
                  (REFERENCE / "compiler/tests/fixtures/stencils/cvd.f90").read_text(),
                  (REFERENCE / "compiler/tests/fixtures/stencils/cdw.f90").read_text())


def stepper_source() -> Source:
    box = REFERENCE / "compiler/tests/apps/box"
    # the module's other dependencies (the boundary and source modules) serve procedures not run here
    stepper = re.sub(r"^\s*use (boundaries|sources).*$", "", (box / "stepper.f90").read_text(), flags=re.M)
    return Source((box / "params.f90").read_text(), stepper)


def jacobi_source() -> Source:
    """The first DO nest inside the sweep loop of relax.f90, verbatim, as a subroutine of its arrays."""
    lines = (REFERENCE / "compiler/tests/apps/relax/relax.f90").read_text().splitlines()
    start = next(n for n, l in enumerate(lines) if re.match(r"\s*do sweep\b", l))
    first = next(n for n in range(start + 1, len(lines)) if re.match(r"\s*do j\b", lines[n]))
    depth, last = 0, first
    for n in range(first, len(lines)):
        text = lines[n].split("!", 1)[0].strip().lower()
        if re.match(r"do\b", text):
            depth += 1
        elif re.match(r"end\s*do\b", text):
            depth -= 1
            if depth == 0:
                last = n
                break
    nest = "\n".join(lines[first:last + 1])
    return Source("module relax_nest\n  integer, parameter :: rp = kind(1d0)\ncontains\n"
                  "subroutine sweep(u, v, n)\n  real(rp), intent(in) :: u(0:, 0:)\n"
                  "  real(rp), intent(inout) :: v(0:, 0:)\n  integer, intent(in) :: n\n  integer :: i, j\n"
                  f"{nest}\nend subroutine sweep\nend module relax_nest\n")


MAIN_PROGRAMS = (("cdu", "cdu.f90", "cdu_main.f90", "cdu_test"), ("cdv", "cvd.f90", "cvd_main.f90", "cdv_test"),
                 ("cdw", "cdw.f90", "cdw_main.f90", "cdw_test"))
MAIN_SIZES = ((16, 16, 16), (12, 10, 8))


def main_program_cases() -> dict:
    """Each test program run as written; the inputs it built and the values it wrote."""
    stencils = REFERENCE / "compiler/tests/fixtures/stencils"
    out = {}
    for n, (nx, ny, nz) in enumerate(MAIN_SIZES):
        defines = {} if (nx, ny, nz) == (16, 16, 16) else {"VAR_NX": nx, "VAR_NY": ny, "VAR_NZ": nz}
        out[f"main{n}_size"] = np.array([nx, ny, nz], dtype=np.float64)
        for which, module, program, unit in MAIN_PROGRAMS:
            src = Source((stencils / module).read_text(), (stencils / program).read_text(), defines=defines)
            out[f"main{n}_{which}"] = np.array(src.run_program(unit))
            arrays = src.program_arrays
            for k in "uvw":
                key = f"main{n}_{k.upper()}"
                if key in out:
                    assert np.array_equal(out[key], arrays[k])  # the three programs build the same inputs
                out[key] = arrays[k]
    return out


def advection_case(src: Source, nx, ny, nz, ghosts, dx, dy, dz, seed) -> dict:
    rng = np.random.default_rng(seed)
    shape = (nz + 2 * ghosts, ny + 2 * ghosts, nx + 2 * ghosts)
    U, V, W = (2.0 * rng.random(shape) - 1.0 for _ in range(3))
    drop = (slice(ghosts - 1, shape[0] - ghosts + 1), slice(ghosts - 1, shape[1] - ghosts + 1),
            slice(ghosts - 1, shape[2] - ghosts + 1))  # what the procedures see: one ghost layer
    inner = (slice(ghosts, ghosts + nz), slice(ghosts, ghosts + ny), slice(ghosts, ghosts + nx))
    out = {"U": U, "V": V, "W": W}
    for name in ("cdu", "cdv", "cdw"):
        o = np.full(shape, np.nan)
        src.call(name, o[drop], U[drop], V[drop], W[drop], dx, dy, dz, nx, ny, nz)
        out[name] = o[inner].copy()
    return out


def procedure_case(src: Source, U, V, W, nx, ny, nz, ghosts, dx, dy, dz, seed) -> dict:
    """Each procedure of the U, V and W trees alone on one-ghost-layer inputs: div after set(0), adv onto
    zeros, multiply(0.5) of div."""
    assert ghosts == 1
    shape = U.shape
    inner = (slice(1, 1 + nz), slice(1, 1 + ny), slice(1, 1 + nx))
    out = {}
    for c in "uvw":
        div = np.full(shape, np.nan)
        src.call("set", div, 0.0, nx, ny, nz)
        src.call(f"cd{c}div", div, U, V, W, dx, dy, dz, nx, ny, nz)
        adv = np.full(shape, np.nan)
        src.call("set", adv, 0.0, nx, ny, nz)
        src.call(f"cd{c}adv", adv, U, V, W, dx, dy, dz, nx, ny, nz)
        half = div.copy()
        src.call("multiply", half, 0.5, nx, ny, nz)
        out[f"cd{c}div"], out[f"cd{c}adv"], out[f"cd{c}half"] = div[inner].copy(), adv[inner].copy(), half[inner].copy()
    return out


def generate() -> dict:
    out = {}
    adv = advection_source()
    for n, case in enumerate(ADVECTION_CASES):
        out[f"adv{n}_case"] = np.array(case, dtype=np.float64)
        for k, v in advection_case(adv, *case).items():
            out[f"adv{n}_{k}"] = v
    for k, v in procedure_case(adv, out["adv0_U"], out["adv0_V"], out["adv0_W"], *ADVECTION_CASES[0]).items():
        out[f"proc_{k}"] = v
    nx, ny, nz, dx, dt, nu, seed = DIFFUSION_CASE
    step = stepper_source()
    step.globals.update(nx=nx, ny=ny, nz=nz, dx=dx, dt=dt, nu=nu)
    a = np.random.default_rng(seed).random((nz + 4, ny + 4, nx + 4))
    b = np.full_like(a, np.nan)
    step.call("diffuse", a, b)
    out["diff_case"] = np.array(DIFFUSION_CASE, dtype=np.float64)
    out["diff_a"], out["diff_b"] = a, b[2:-2, 2:-2, 2:-2].copy()
    n, seed = JACOBI_CASE
    u = np.random.default_rng(seed).random((n + 2, n + 2))
    v = np.full_like(u, np.nan)
    jacobi_source().call("sweep", u, v, n)
    out["jac_case"] = np.array(JACOBI_CASE, dtype=np.float64)
    out["jac_u"], out["jac_v"] = u, v[1:-1, 1:-1].copy()
    out.update(main_program_cases())
    return out


def main():
    np.savez_compressed(OUT, **generate())


if __name__ == "__main__":
    main()
