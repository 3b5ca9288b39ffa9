"""Parity of the fused sm_103a advection launch with the C oracle, through the kernel C ABI.

Bar: bit-identical FP64 (the kernels are built with --fmad=false and keep the
reference's expression grouping). Sizes cover the reference driver's geometry
(one ghost layer, dx = 1/N), the restated driver's (halo 2, 10/10/5 m), odd and
one-cell extents, pitched strides and the Euler advance mode.
"""

import numpy as np
import pytest

from compiler import native
from compiler import workloads as wl
from oracle import api, literal

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def _device(torch, a, pitch=None):
    """Copy a host array to the device, optionally into a wider (pitched) x stride."""
    nz, ny, nx = a.shape
    if pitch is None:
        return torch.from_numpy(a).cuda(), nx
    t = torch.full((nz, ny, pitch), float("nan"), dtype=torch.float64, device="cuda")
    t[:, :, :nx] = torch.from_numpy(a).cuda()
    return t, pitch


def _run(torch, fields: wl.Fields, mode=native.TENDENCY, dt=0.0, pitch=None, which=("U", "V", "W"),
         variant=native.FACES, scalars=True):
    geo = fields.geometry
    ins = [_device(torch, a, pitch)[0] for a in fields.arrays()]
    sx = ins[0].shape[2]
    outs = [torch.full_like(t, float("nan")) for t in ins]
    grid = native.make_grid(geo.nx, geo.ny, geo.nz, geo.halo, geo.dx, geo.dy, geo.dz, sx=sx)
    ptr = [t.data_ptr() for t in ins]
    optr = [t.data_ptr() for t in outs]
    sel = [optr[n] if name in which else None for n, name in enumerate(("U", "V", "W"))]
    native.advection(grid, *ptr[:3], *sel, scalars=ptr[3:] if scalars else (),
                     scalar_out=optr[3:] if scalars else (), mode=mode, dt=dt, variant=variant)
    torch.cuda.synchronize()
    nx = geo.nx + 2 * geo.halo
    return [o[:, :, :nx].cpu().numpy() for o in outs]


def _oracle(fields: wl.Fields, mode=native.TENDENCY, dt=0.0):
    geo = fields.geometry
    t = api.advection_step({"U": fields.U, "V": fields.V, "W": fields.W}, geo.dx, geo.dy, geo.dz, geo.halo,
                           fields.scalars)
    out = [t["U"], t["V"], t["W"], *[t[f"S{n}"] for n in range(len(fields.scalars))]]
    if mode == native.ADVANCE:
        out = [api.euler(a.copy(), o, dt, geo.halo) for a, o in zip(fields.arrays(), out)]
    return out


def _interior(a, geo):
    return a[geo.interior()]


VARIANTS = [native.FACES, native.DIRECT]


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("shape,halo,nscalar", [((3, 5, 2), 1, 0), ((1, 1, 1), 1, 1), ((12, 10, 6), 2, 3),
                                                ((33, 9, 17), 2, 2), ((64, 64, 32), 2, 1), ((40, 17, 70), 2, 4),
                                                ((65, 24, 33), 1, 3)])
def test_tendencies_bit_exact(cuda, shape, halo, nscalar, variant):
    geo = wl.Geometry(*shape, halo=halo)
    fields = wl.advection_fields(geo, seed=0, nscalar=nscalar)
    got = _run(cuda, fields, variant=variant)
    ref = _oracle(fields)
    for g, r in zip(got, ref):
        assert np.array_equal(_bits(_interior(g, geo)), _bits(_interior(r, geo)))


def test_full_size_step_bit_exact(cuda):
    """The measured workload itself (512 x 512 x 128, halo 2, U, V, W and 3 scalars): every output bit-identical
    to the C oracle, and a constant field still gives an exactly zero tendency at this size."""
    geo = wl.Geometry(512, 512, 128, halo=2, dx=10.0, dy=10.0, dz=5.0)
    fields = wl.advection_fields(geo, seed=0, nscalar=3)
    got = _run(cuda, fields)
    ref = _oracle(fields)
    for g, r in zip(got, ref):
        assert np.array_equal(_bits(_interior(g, geo)), _bits(_interior(r, geo)))
    del got, ref
    flat = wl.Fields(geo, np.full_like(fields.U, 3.0), np.full_like(fields.V, -2.0), np.full_like(fields.W, 0.5),
                     [np.full_like(fields.U, 7.0)])
    for g in _run(cuda, flat):
        assert not np.any(_interior(g, geo))


@pytest.mark.parametrize("variant", VARIANTS)
def test_reference_driver_geometry(cuda, variant):
    fields = wl.reference_driver_fields(16, 12, 10, seed=7)
    geo = fields.geometry
    got = _run(cuda, fields, variant=variant)
    ref = _oracle(fields)
    for g, r in zip(got, ref):
        assert np.array_equal(_bits(_interior(g, geo)), _bits(_interior(r, geo)))


def test_cdu_main_fixture_inputs_against_literal(cuda):
    """The sin/cos inputs of cdu_main.f90:38-50 at 16^3, checked against the literal transcription."""
    U, V, W, dx, dy, dz = literal.fixture_inputs(16, 16, 16)
    geo = wl.Geometry(16, 16, 16, halo=1, dx=dx, dy=dy, dz=dz)
    fields = wl.Fields(geo, U, V, W, [])
    got = _run(cuda, fields)
    for g, which, arr in zip(got, ("cdu", "cdv", "cdw"), (U, V, W)):
        ref = literal.tendency(which, np.zeros_like(U), U, V, W, dx, dy, dz)
        assert np.array_equal(_bits(_interior(g, geo)), _bits(_interior(ref, geo)))


def test_pitched_rows(cuda):
    geo = wl.Geometry(13, 7, 5, halo=2)
    fields = wl.advection_fields(geo, seed=3, nscalar=1)
    got = _run(cuda, fields, pitch=geo.nx + 2 * geo.halo + 5)
    ref = _oracle(fields)
    for g, r in zip(got, ref):
        assert np.array_equal(_bits(_interior(g, geo)), _bits(_interior(r, geo)))


@pytest.mark.parametrize("variant", VARIANTS)
def test_advance_mode(cuda, variant):
    geo = wl.Geometry(20, 18, 9, halo=2)
    fields = wl.advection_fields(geo, seed=5, nscalar=2)
    got = _run(cuda, fields, mode=native.ADVANCE, dt=0.1, variant=variant)
    ref = _oracle(fields, mode=native.ADVANCE, dt=0.1)
    for g, r in zip(got, ref):
        assert np.array_equal(_bits(_interior(g, geo)), _bits(_interior(r, geo)))


@pytest.mark.parametrize("which", [("U",), ("V",), ("W",), ("U", "W"), ("V", "W"), ()])
def test_subset_of_outputs_leaves_others_untouched(cuda, which):
    geo = wl.Geometry(37, 11, 35, halo=2)
    fields = wl.advection_fields(geo, seed=2, nscalar=2 if not which else 0)
    got = _run(cuda, fields, which=which)
    ref = _oracle(fields)
    for n, name in enumerate(("U", "V", "W")):
        if name in which:
            assert np.array_equal(_bits(_interior(got[n], geo)), _bits(_interior(ref[n], geo)))
        else:
            assert np.isnan(got[n]).all()
    for g, r in zip(got[3:], ref[3:]):
        assert np.array_equal(_bits(_interior(g, geo)), _bits(_interior(r, geo)))


def test_exact_half_on_small_values(cuda):
    """Tendencies of tiny fields exercise the integer halving on subnormal and smallest-normal results."""
    geo = wl.Geometry(9, 7, 5, halo=1, dx=1.0, dy=1.0, dz=1.0)
    rng = np.random.default_rng(3)
    scale = np.float64(2.0) ** -537
    arrays = [rng.normal(size=geo.shape) * scale for _ in range(3)]
    arrays[0][2, 3, 4] = 0.0
    fields = wl.Fields(geo, *arrays, [])
    got = _run(cuda, fields)
    ref = _oracle(fields)
    assert any((np.abs(_interior(r, geo)) < np.finfo(np.float64).tiny).any() for r in ref)
    for g, r in zip(got, ref):
        assert np.array_equal(_bits(_interior(g, geo)), _bits(_interior(r, geo)))


@pytest.mark.parametrize("shape,halo", [((12, 10, 6), 2), ((5, 4, 3), 1), ((9, 7, 4), 3)])
def test_halo_fill_bit_exact(cuda, shape, halo):
    geo = wl.Geometry(*shape, halo=halo)
    rng = np.random.default_rng(11)
    arrays = [rng.normal(size=geo.shape) for _ in range(3)]
    kinds = [0, 1, 0]
    dev = [cuda.from_numpy(a).cuda() for a in arrays]
    grid = native.make_grid(geo.nx, geo.ny, geo.nz, halo, geo.dx, geo.dy, geo.dz)
    native.halo_fill(grid, [t.data_ptr() for t in dev], kinds)
    cuda.cuda.synchronize()
    for a, kind, t in zip(arrays, kinds, dev):
        ref = api.halo(a.copy(), kind, halo)
        assert np.array_equal(_bits(t.cpu().numpy()), _bits(ref))


def test_argument_errors(cuda):
    geo = wl.Geometry(4, 4, 4, halo=1)
    t = cuda.zeros(geo.shape, dtype=cuda.float64, device="cuda")
    grid = native.make_grid(4, 4, 4, 1, 1.0, 1.0, 1.0)
    with pytest.raises(native.NativeError) as err:
        native.advection(grid, t.data_ptr(), t.data_ptr(), t.data_ptr(), ut=t.data_ptr())
    assert err.value.status == 3
    bad = native.make_grid(4, 4, 4, 1, 1.0, 1.0, 1.0, sx=3)
    with pytest.raises(native.NativeError):
        native.advection(bad, t.data_ptr(), t.data_ptr(), t.data_ptr())


def test_golden_fixtures_on_the_gpu(cuda):
    from pathlib import Path

    z = np.load(Path(__file__).with_name("golden") / "advection_small.npz")
    dx, dy, dz = (float(v) for v in z["spacing"])
    nz, ny, nx = (s - 2 for s in z["U"].shape)
    geo = wl.Geometry(nx, ny, nz, halo=1, dx=dx, dy=dy, dz=dz)
    got = _run(cuda, wl.Fields(geo, z["U"], z["V"], z["W"], []))
    for g, which in zip(got, ("cdu", "cdv", "cdw")):
        assert np.array_equal(_bits(_interior(g, geo)), _bits(_interior(z[which], geo)))
    ins = [z[f"h2_in{n}"] for n in range(6)]
    geo2 = wl.Geometry(12, 10, 6, halo=2)
    got = _run(cuda, wl.Fields(geo2, *ins[:3], ins[3:]))
    for n, g in enumerate(got):
        assert np.array_equal(_bits(_interior(g, geo2)), _bits(_interior(z[f"h2_tend{n}"], geo2)))


@pytest.mark.parametrize("component", [0, 1, 2])
def test_procedure_launch_chain_equals_fused(cuda, component):
    """set, div, adv, multiply(0.5) as four launches gives the fused launch's bits."""
    geo = wl.Geometry(41, 23, 19, halo=2)
    fields = wl.advection_fields(geo, seed=4)
    ins = [cuda.from_numpy(a).cuda() for a in fields.arrays()]
    chained = cuda.full_like(ins[0], 5.0)
    grid = native.make_grid(geo.nx, geo.ny, geo.nz, geo.halo, geo.dx, geo.dy, geo.dz)
    u, v, w = (t.data_ptr() for t in ins)
    div, adv = [(native.CDU_DIV, native.CDU_ADV), (native.CDV_DIV, native.CDV_ADV),
                (native.CDW_DIV, native.CDW_ADV)][component]
    native.procedure(native.SET, grid, chained.data_ptr(), value=0.0)
    native.procedure(div, grid, chained.data_ptr(), u, v, w)
    native.procedure(adv, grid, chained.data_ptr(), u, v, w)
    native.procedure(native.MULTIPLY, grid, chained.data_ptr(), value=0.5)
    cuda.cuda.synchronize()
    got = _run(cuda, fields)[component]
    assert np.array_equal(_bits(_interior(chained.cpu().numpy(), geo)), _bits(_interior(got, geo)))
