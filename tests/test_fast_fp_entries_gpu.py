"""Generated entries under the fast-fp contract, through the C ABI as the spliced call blocks drive them.

A resident build prepared with --fast-fp (the reference's option,
compiler/resident/__main__.py:34-35 and compiler/resident/build.py:22,66-67)
opens its contexts with FORT_SCOPE_NUMERICS_FAST; the entries that have a
fast-fp kernel then run it. These tests drive the fused momentum procedures,
the advection step (whole and as a slab pipeline) and the Euler advance through
a domain in that contract and compare with the oracle within the tolerance of
tests/tolerance.py; a context switched back to strict is bit-exact again.
"""

import numpy as np
import pytest
import tolerance

from compiler import emission, native
from compiler import workloads as wl
from compiler.resident.domain import ResidentDomain
from compiler.runtime import abi
from oracle import api

pytestmark = pytest.mark.gpu


@pytest.fixture()
def fast_domain(cuda):
    lib = native.runtime()
    dom = ResidentDomain(lib, fast_fp=True)
    yield dom, emission.bind(lib)
    if dom.context:
        dom.close()


def _call(fns, dom, procedure, arrays, reals=(), ints=()):
    return emission.call(fns, procedure, dom.context, abi.GPU, arrays, reals, ints)


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


@pytest.mark.parametrize("which", ["cdu", "cdv", "cdw"])
def test_fast_procedure_entries(fast_domain, which):
    dom, fns = fast_domain
    f = wl.reference_driver_fields(40, 20, 12, seed=3)
    geo = f.geometry
    out = np.zeros_like(f.U)
    dom.begin_epoch()
    handles = [dom.bind_real64(a) for a in (out, f.U, f.V, f.W)]
    for _ in range(3):
        assert _call(fns, dom, f"momentumadvection::{which}", handles, [geo.dx, geo.dy, geo.dz],
                     [geo.nx, geo.ny, geo.nz]) == abi.OK
        assert dom.lib.fort_scope_graph_flush_v1(dom.context) == abi.OK
    dom.end_epoch()
    ref = api.momentum(which, np.zeros_like(f.U), f.U, f.V, f.W, geo.dx, geo.dy, geo.dz, 1)
    tolerance.check(out[geo.interior()], ref[geo.interior()], which)
    ghost = out.copy()
    ghost[geo.interior()] = 0.0
    assert not ghost.any()


def test_fast_step_entry_and_switch_back_to_strict(fast_domain):
    dom, fns = fast_domain
    geo = wl.Geometry(64, 64, 32, halo=2)
    f = wl.advection_fields(geo, seed=0, nscalar=3)
    fast = [np.zeros_like(f.U) for _ in range(6)]
    strict = [np.zeros_like(f.U) for _ in range(6)]
    dom.begin_epoch()
    h_in = [dom.bind_real64(a) for a in f.arrays()]
    h_fast = [dom.bind_real64(a) for a in fast]
    h_strict = [dom.bind_real64(a) for a in strict]
    spacing, grid = [geo.dx, geo.dy, geo.dz], [geo.nx, geo.ny, geo.nz, geo.halo]
    assert _call(fns, dom, "advection::step3", [*h_fast[:3], *h_in, *h_fast[3:]], spacing, grid) == abi.OK
    assert dom.lib.fort_scope_numerics_set_v1(dom.context, abi.NUMERICS_STRICT) == abi.OK
    assert _call(fns, dom, "advection::step3", [*h_strict[:3], *h_in, *h_strict[3:]], spacing, grid) == abi.OK
    dom.end_epoch()
    ref = api.advection_step({"U": f.U, "V": f.V, "W": f.W}, geo.dx, geo.dy, geo.dz, geo.halo, f.scalars)
    inner = geo.interior()
    differs = 0
    for got_fast, got_strict, name in zip(fast, strict, ["U", "V", "W", "S0", "S1", "S2"]):
        tolerance.check(got_fast[inner], ref[name][inner], name)
        assert np.array_equal(_bits(got_strict[inner]), _bits(ref[name][inner]))
        differs += not np.array_equal(_bits(got_fast[inner]), _bits(ref[name][inner]))
    assert differs  # the fast kernel ran: its rounding differs from the strict contract


def test_fast_step_as_slab_pipeline(fast_domain):
    """A step the host rewrites and reads every round runs as z-slabs (uploads, kernels and publications
    overlapped); under the fast contract each slab runs the fast kernel."""
    dom, fns = fast_domain
    geo = wl.Geometry(96, 80, 96, halo=2)
    f = wl.advection_fields(geo, seed=4, nscalar=1)
    inputs = [a.copy() for a in f.arrays()]
    outputs = [np.zeros_like(a) for a in inputs]
    dom.begin_epoch()
    h_in = [dom.bind_real64(a) for a in inputs]
    h_out = [dom.bind_real64(a) for a in outputs]
    arrays = [*h_out[:3], *h_in[:3], *h_in[3:], *h_out[3:]]
    for _ in range(4):
        dom.host_modify(h_in)
        assert _call(fns, dom, "advection::step1", arrays, [geo.dx, geo.dy, geo.dz],
                     [geo.nx, geo.ny, geo.nz, geo.halo]) == abi.OK
        dom.observe(h_out)
    dom.end_epoch()
    ref = api.advection_step({"U": f.U, "V": f.V, "W": f.W}, geo.dx, geo.dy, geo.dz, geo.halo, f.scalars)
    inner = geo.interior()
    for got, name in zip(outputs, ["U", "V", "W", "S0"]):
        tolerance.check(got[inner], ref[name][inner], name)


def test_fast_ten_euler_steps_with_boundary_fill(fast_domain):
    dom, fns = fast_domain
    geo = wl.Geometry(64, 64, 32, halo=2)
    f = wl.advection_fields(geo, seed=0, nscalar=1)
    dt = 0.1
    a = [x.copy() for x in f.arrays()]
    b = [np.zeros_like(x) for x in a]
    dom.begin_epoch()
    ha = [dom.bind_real64(x) for x in a]
    hb = [dom.bind_real64(x) for x in b]
    grid = [geo.nx, geo.ny, geo.nz, geo.halo]
    for _ in range(10):
        arrays = [*hb[:3], *ha[:3], *ha[3:], *hb[3:]]
        assert _call(fns, dom, "advection::advance1", arrays, [geo.dx, geo.dy, geo.dz, dt], grid) == abi.OK
        assert _call(fns, dom, "advection::halo1", hb, [], grid) == abi.OK
        ha, hb = hb, ha
    dom.end_epoch()
    state = [x.copy() for x in f.arrays()]
    for _ in range(10):
        t = api.advection_step({"U": state[0], "V": state[1], "W": state[2]}, geo.dx, geo.dy, geo.dz, geo.halo,
                               state[3:])
        new = [api.euler(x.copy(), t[name], dt, geo.halo) for x, name in zip(state, ["U", "V", "W", "S0"])]
        for n, x in enumerate(new):
            api.halo(x, 1 if n == 2 else 0, geo.halo)
        state = new
    for got, want, name in zip(a, state, ["U", "V", "W", "S0"]):
        tolerance.check(got, want, name)
