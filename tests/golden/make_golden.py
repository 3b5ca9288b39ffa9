"""Writes tests/golden/advection_small.npz: small known-answer fixtures of the advection path.

Inputs: the deterministic sin/cos formula of the reference's stencil fixtures
(compiler/tests/fixtures/stencils/cdu_main.f90:38-50) at 10 x 8 x 6, stored
as computed (so the platform's libm does not enter the check), plus a seeded
halo-2 sine-mode set with three scalars. Outputs: CDU, CDV and CDW by the
literal Python transcription of the Fortran (oracle/literal.py), scalar
tendencies, one Euler step and the boundary fill by the C oracle. Run from the
repository root: python tests/golden/make_golden.py
"""

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT), str(ROOT / "fortran-to-cuda_gb300")]

from compiler import workloads as wl  # noqa: E402
from oracle import api, literal  # noqa: E402


def main():
    U, V, W, dx, dy, dz = literal.fixture_inputs(10, 8, 6)
    out = {"U": U, "V": V, "W": W, "spacing": np.array([dx, dy, dz])}
    for which in ("cdu", "cdv", "cdw"):
        out[which] = literal.tendency(which, np.zeros_like(U), U, V, W, dx, dy, dz)
    geo = wl.Geometry(12, 10, 6, halo=2)
    f = wl.advection_fields(geo, seed=0, nscalar=3)
    for n, a in enumerate(f.arrays()):
        out[f"h2_in{n}"] = a
    t = api.advection_step({"U": f.U, "V": f.V, "W": f.W}, geo.dx, geo.dy, geo.dz, geo.halo, f.scalars)
    for n, name in enumerate(["U", "V", "W", "S0", "S1", "S2"]):
        out[f"h2_tend{n}"] = t[name]
        step = api.euler(f.arrays()[n].copy(), t[name], 0.1, geo.halo)
        out[f"h2_euler{n}"] = api.halo(step, 1 if n == 2 else 0, geo.halo)
    np.savez_compressed(Path(__file__).with_name("advection_small.npz"), **out)


if __name__ == "__main__":
    main()
