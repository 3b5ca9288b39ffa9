"""The fast-fp advection kernel (F2C_KERNEL_FAST) against the C oracle, through the kernel C ABI.

The fast kernel is the counterpart of the reference's --fast-fp build
(compiler/resident/build.py:22): FMA contraction and a regrouped form of the
same tendencies. Its results differ from the oracle (the reference's strict
arithmetic) by rounding only. Bar, per field: max |fast - oracle| over the
interior <= 1e-12 * max |oracle| (normwise relative error). The pointwise
relative error, |d| / max(|oracle|, 1e-300), is reported and bounded where the
oracle is not itself a cancellation residue (|oracle| >= 1e-3 of the field's
maximum).
"""

import numpy as np
import pytest
import tolerance

from compiler import native
from compiler import workloads as wl
from oracle import api

pytestmark = pytest.mark.gpu


def _run(torch, fields, mode=native.TENDENCY, dt=0.0, which=("U", "V", "W"), scalars=True, pitch=None):
    geo = fields.geometry
    ins = []
    for a in fields.arrays():
        t = torch.from_numpy(a).cuda()
        if pitch is not None:
            wide = torch.full((a.shape[0], a.shape[1], pitch), float("nan"), dtype=torch.float64, device="cuda")
            wide[:, :, :a.shape[2]] = t
            t = wide
        ins.append(t)
    outs = [torch.full_like(t, float("nan")) for t in ins]
    grid = native.make_grid(geo.nx, geo.ny, geo.nz, geo.halo, geo.dx, geo.dy, geo.dz, sx=ins[0].shape[2])
    ptr = [t.data_ptr() for t in ins]
    optr = [t.data_ptr() for t in outs]
    sel = [optr[n] if name in which else None for n, name in enumerate(("U", "V", "W"))]
    native.advection(grid, *ptr[:3], *sel, scalars=ptr[3:] if scalars else (),
                     scalar_out=optr[3:] if scalars else (), mode=mode, dt=dt, variant=native.FAST)
    torch.cuda.synchronize()
    ex = geo.nx + 2 * geo.halo
    return [o[:, :, :ex].cpu().numpy() for o in outs]


def _oracle(fields, mode=native.TENDENCY, dt=0.0):
    geo = fields.geometry
    t = api.advection_step({"U": fields.U, "V": fields.V, "W": fields.W}, geo.dx, geo.dy, geo.dz, geo.halo,
                           fields.scalars)
    out = [t["U"], t["V"], t["W"], *[t[f"S{n}"] for n in range(len(fields.scalars))]]
    if mode == native.ADVANCE:
        out = [api.euler(a.copy(), o, dt, geo.halo) for a, o in zip(fields.arrays(), out)]
    return out


def _check(got, ref, geo, names):
    inner = geo.interior()
    for name, g, r in zip(names, got, ref):
        tolerance.check(g[inner], r[inner], name)


@pytest.mark.parametrize("shape,halo,nscalar", [((3, 5, 2), 1, 0), ((1, 1, 1), 1, 1), ((12, 10, 6), 2, 3),
                                                ((33, 9, 17), 2, 2), ((64, 64, 32), 2, 1), ((40, 17, 70), 2, 4),
                                                ((65, 24, 33), 1, 3), ((96, 41, 5), 2, 0)])
def test_fast_tendencies_within_tolerance(cuda, shape, halo, nscalar):
    geo = wl.Geometry(*shape, halo=halo)
    fields = wl.advection_fields(geo, seed=1, nscalar=nscalar)
    got = _run(cuda, fields)
    ref = _oracle(fields)
    _check(got, ref, geo, ["U", "V", "W", *[f"S{n}" for n in range(nscalar)]])


@pytest.mark.parametrize("which", [("U",), ("V",), ("W",), ("U", "W"), ()])
def test_fast_single_components(cuda, which):
    """One momentum component alone (the CDU, CDV and CDW entries), two of three, and scalars alone."""
    geo = wl.Geometry(37, 19, 21, halo=2)
    fields = wl.advection_fields(geo, seed=5, nscalar=2)
    got = _run(cuda, fields, which=which)
    ref = _oracle(fields)
    names = ["U", "V", "W", "S0", "S1"]
    keep = [n for n, name in enumerate(names) if name in which or name.startswith("S")]
    _check([got[n] for n in keep], [ref[n] for n in keep], geo, [names[n] for n in keep])
    for n, name in enumerate(names[:3]):
        if name not in which:
            assert np.isnan(got[n]).all(), f"{name} was written although not requested"


def test_fast_advance_mode(cuda):
    geo = wl.Geometry(45, 30, 24, halo=2)
    fields = wl.advection_fields(geo, seed=2, nscalar=3)
    got = _run(cuda, fields, mode=native.ADVANCE, dt=0.1)
    ref = _oracle(fields, mode=native.ADVANCE, dt=0.1)
    _check(got, ref, geo, ["U", "V", "W", "S0", "S1", "S2"])


def test_fast_pitched_rows_and_reference_geometry(cuda):
    geo = wl.Geometry(13, 7, 5, halo=2)
    fields = wl.advection_fields(geo, seed=3, nscalar=1)
    got = _run(cuda, fields, pitch=geo.nx + 2 * geo.halo + 5)
    _check(got, _oracle(fields), geo, ["U", "V", "W", "S0"])
    fields = wl.reference_driver_fields(16, 12, 10, seed=7)
    got = _run(cuda, fields)
    _check(got, _oracle(fields), fields.geometry, ["U", "V", "W"])


def test_fast_constant_fields_give_rounding_level_tendency(cuda):
    """Constant fields: the exact tendency is zero; the FMA form leaves at most the rounding residue of one
    product per direction (|t| <= 4 ulp of the largest term A*|U|*|V|*16)."""
    geo = wl.Geometry(40, 24, 12, halo=2)
    shape = geo.shape
    flat = wl.Fields(geo, np.full(shape, 3.0), np.full(shape, -2.0), np.full(shape, 0.5), [np.full(shape, 7.0)])
    bound = 4 * np.finfo(np.float64).eps * (0.25 / min(geo.dx, geo.dy, geo.dz)) * 16 * 3.0 * 3.0 * 7.0
    for g in _run(cuda, flat):
        assert np.abs(g[geo.interior()]).max() <= bound


def test_fast_full_size_step(cuda):
    """The measured workload (512 x 512 x 128, halo 2, U, V, W and 3 scalars) within the tolerance."""
    geo = wl.Geometry(512, 512, 128, halo=2, dx=10.0, dy=10.0, dz=5.0)
    fields = wl.advection_fields(geo, seed=0, nscalar=3)
    got = _run(cuda, fields)
    ref = _oracle(fields)
    _check(got, ref, geo, ["U", "V", "W", "S0", "S1", "S2"])
