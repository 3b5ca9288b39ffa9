"""Generated numerical entries through the C ABI, driven like the spliced Fortran call blocks.

Each test opens an epoch on a residency domain, binds host arrays, calls the
entries (``cpp_fort_shared_<digest>``) with FORT_SCOPE_GPU exactly as the
call block does (context, mode, handles, scalars by reference), publishes,
and compares the host arrays with the C oracle bit for bit.
"""

import numpy as np
import pytest

from compiler import emission, native
from compiler import workloads as wl
from compiler.resident.domain import ResidentDomain
from compiler.runtime import abi
from oracle import api

pytestmark = pytest.mark.gpu


@pytest.fixture()
def resident(cuda):
    lib = native.runtime()
    dom = ResidentDomain(lib)
    yield dom, emission.bind(lib)
    if dom.context:
        dom.close()


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def _same(a, b):
    return np.array_equal(_bits(a), _bits(b))


def _call(fns, dom, procedure, arrays, reals=(), ints=()):
    return emission.call(fns, procedure, dom.context, abi.GPU, arrays, reals, ints)


@pytest.mark.parametrize("which", ["cdu", "cdv", "cdw"])
def test_procedure_entry_matches_oracle(resident, which):
    dom, fns = resident
    f = wl.reference_driver_fields(24, 20, 12, seed=3)
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
    assert _same(out[geo.interior()], ref[geo.interior()])
    ghost = out.copy()
    ghost[geo.interior()] = 0.0
    assert not ghost.any()  # the ghost layer of the output is untouched
    g = dom.graph_stats()
    assert (g.instantiations, g.replays) == (1, 1)


@pytest.mark.parametrize("which", ["cdu", "cdv", "cdw"])
def test_four_procedure_chain_equals_fused_entry(resident, which):
    dom, fns = resident
    f = wl.reference_driver_fields(33, 17, 9, seed=5)
    geo = f.geometry
    chained, fused = np.full_like(f.U, 7.0), np.zeros_like(f.U)
    dom.begin_epoch()
    hc, hf, hu, hv, hw = (dom.bind_real64(a) for a in (chained, fused, f.U, f.V, f.W))
    spacing = [geo.dx, geo.dy, geo.dz]
    n = [geo.nx, geo.ny, geo.nz]
    assert _call(fns, dom, "momentumadvection::set", [hc], [0.0], n) == abi.OK
    assert _call(fns, dom, f"momentumadvection::{which}div", [hc, hu, hv, hw], spacing, n) == abi.OK
    assert _call(fns, dom, f"momentumadvection::{which}adv", [hc, hu, hv, hw], spacing, n) == abi.OK
    assert _call(fns, dom, "momentumadvection::multiply", [hc], [0.5], n) == abi.OK
    assert _call(fns, dom, f"momentumadvection::{which}", [hf, hu, hv, hw], spacing, n) == abi.OK
    dom.end_epoch()
    inner = geo.interior()
    assert _same(chained[inner], fused[inner])
    ref = api.momentum(which, np.zeros_like(f.U), f.U, f.V, f.W, geo.dx, geo.dy, geo.dz, 1)
    assert _same(fused[inner], ref[inner])


def test_step_entry_with_scalars(resident):
    dom, fns = resident
    geo = wl.Geometry(64, 64, 32, halo=2)
    f = wl.advection_fields(geo, seed=0, nscalar=3)
    outs = [np.zeros_like(f.U) for _ in range(6)]
    dom.begin_epoch()
    h_out = [dom.bind_real64(a) for a in outs]
    h_in = [dom.bind_real64(a) for a in f.arrays()]
    arrays = [*h_out[:3], *h_in[:3], *h_in[3:], *h_out[3:]]
    assert _call(fns, dom, "advection::step3", arrays, [geo.dx, geo.dy, geo.dz],
                 [geo.nx, geo.ny, geo.nz, geo.halo]) == abi.OK
    dom.end_epoch()
    ref = api.advection_step({"U": f.U, "V": f.V, "W": f.W}, geo.dx, geo.dy, geo.dz, geo.halo, f.scalars)
    inner = geo.interior()
    for got, name in zip(outs, ["U", "V", "W", "S0", "S1", "S2"]):
        assert _same(got[inner], ref[name][inner])


@pytest.mark.parametrize("nscalar", [0, 1, 3])
def test_ten_euler_steps_with_boundary_fill(resident, nscalar):
    """The 64x64x32 configuration: 10 steps at dt = 0.1, forward Euler, periodic x/y, walls in z."""
    dom, fns = resident
    geo = wl.Geometry(64, 64, 32, halo=2)
    f = wl.advection_fields(geo, seed=0, nscalar=nscalar)
    dt = 0.1
    a = [x.copy() for x in f.arrays()]
    b = [np.zeros_like(x) for x in a]
    dom.begin_epoch()
    ha = [dom.bind_real64(x) for x in a]
    hb = [dom.bind_real64(x) for x in b]
    grid = [geo.nx, geo.ny, geo.nz, geo.halo]
    for _ in range(10):
        arrays = [*hb[:3], *ha[:3], *ha[3:], *hb[3:]]
        assert _call(fns, dom, f"advection::advance{nscalar}", arrays, [geo.dx, geo.dy, geo.dz, dt], grid) == 0
        assert _call(fns, dom, f"advection::halo{nscalar}", hb, [], grid) == abi.OK
        ha, hb = hb, ha
    dom.end_epoch()
    # reference: the oracle steps the same recipe
    state = [x.copy() for x in f.arrays()]
    for _ in range(10):
        t = api.advection_step({"U": state[0], "V": state[1], "W": state[2]}, geo.dx, geo.dy, geo.dz, geo.halo,
                               state[3:])
        names = ["U", "V", "W", *[f"S{n}" for n in range(nscalar)]]
        new = [api.euler(x.copy(), t[name], dt, geo.halo) for x, name in zip(state, names)]
        for n, x in enumerate(new):
            api.halo(x, 1 if n == 2 else 0, geo.halo)
        state = new
    final = a  # after an even number of steps the newest values are in the first buffer set
    for got, want in zip(final, state):
        assert _same(got, want)


def test_native_mode_and_argument_errors(resident):
    dom, fns = resident
    f = wl.reference_driver_fields(8, 8, 8, seed=1)
    geo = f.geometry
    out = np.zeros_like(f.U)
    dom.begin_epoch()
    hs = [dom.bind_real64(x) for x in (out, f.U, f.V, f.W)]
    spacing, n = [geo.dx, geo.dy, geo.dz], [geo.nx, geo.ny, geo.nz]
    assert emission.call(fns, "momentumadvection::cdu", dom.context, abi.NATIVE, hs, spacing, n) == abi.DECLINED
    assert emission.call(fns, "momentumadvection::cdu", dom.context, 5, hs, spacing, n) == abi.ARGUMENT
    assert _call(fns, dom, "momentumadvection::cdu", [hs[1], hs[1], hs[2], hs[3]], spacing, n) == abi.ALIAS
    assert _call(fns, dom, "momentumadvection::cdu", hs, spacing, [geo.nx + 1, geo.ny, geo.nz]) == abi.ARGUMENT
    assert _call(fns, dom, "momentumadvection::cdu", hs, spacing, [0, geo.ny, geo.nz]) == abi.OK  # no iterations
    flat = np.zeros((4, 4))
    hflat = dom.bind_real64(flat)
    assert _call(fns, dom, "momentumadvection::cdu", [hflat, *hs[1:]], spacing, n) == abi.ARGUMENT
    other = np.zeros((geo.nz + 3, geo.ny + 2, geo.nx + 2))
    hother = dom.bind_real64(other)
    assert _call(fns, dom, "momentumadvection::cdu", [hother, *hs[1:]], spacing, n) == abi.DECLINED
    dom.end_epoch()


def test_budget_too_small_declines_before_any_work(cuda, capfd):
    lib = native.runtime()
    dom = ResidentDomain(lib)
    fns = emission.bind(lib)
    f = wl.reference_driver_fields(16, 16, 16, seed=2)
    geo = f.geometry
    out = np.full_like(f.U, 3.0)
    dom.begin_epoch(budget=2 * f.U.nbytes)
    hs = [dom.bind_real64(x) for x in (out, f.U, f.V, f.W)]
    for _ in range(2):
        assert _call(fns, dom, "momentumadvection::cdu", hs, [geo.dx, geo.dy, geo.dz],
                     [geo.nx, geo.ny, geo.nz]) == abi.DECLINED
    dom.end_epoch()
    dom.close()
    assert (out == 3.0).all()
    assert capfd.readouterr().err.count("Resident domain: the arrays in use exceed the device budget of "
                                        f"{2 * f.U.nbytes} bytes; loop nests whose arrays do not fit together run "
                                        "on the host.") == 1


@pytest.mark.parametrize("nx, ny, nz, path", [(96, 64, 16, "in place"), (96, 64, 48, "in place"),
                                              (512, 512, 24, "slabs"), (300, 200, 90, "slabs")])
def test_arrays_the_host_rewrites_every_step_are_streamed(resident, nx, ny, nz, path):
    """Host writes the inputs and reads the outputs between every step. After two such rounds the runtime
    either hands the kernel the mapped host arrays (a step less than two slabs deep: no copies at all) or
    cuts the step into slabs of about 2.5 M points (10 levels of 512 x 512, thin first and last slabs)
    whose uploads, kernels and publications overlap on three streams. Results stay bit-identical to the
    oracle either way."""
    dom, fns = resident
    geo = wl.Geometry(nx, ny, nz, halo=2)  # arrays of 1 MiB or more are pinned
    f = wl.advection_fields(geo, seed=8, nscalar=1)
    ins = [a.copy() for a in f.arrays()]
    outs = [np.zeros_like(a) for a in ins]
    dom.begin_epoch()
    h_in = [dom.bind_real64(a) for a in ins]
    h_out = [dom.bind_real64(a) for a in outs]
    arrays = [*h_out[:3], *h_in[:3], h_in[3], h_out[3]]
    interior_bytes = sum(8 * geo.nx * geo.ny * geo.nz for _ in outs)
    for step in range(5):
        scale = 1.0 + 0.25 * step
        dom.host_modify(h_in)
        for a, src in zip(ins, f.arrays()):
            a[...] = src * scale
        before = dom.stats()
        assert _call(fns, dom, "advection::step1", arrays, [geo.dx, geo.dy, geo.dz],
                     [geo.nx, geo.ny, geo.nz, geo.halo]) == abi.OK
        called = dom.stats()
        dom.observe(h_out)
        after = dom.stats()
        if path == "slabs" and step >= 1:
            # published slab by slab inside the call (one copy per slab and output), nothing left for the observation
            slabs = called.launches - before.launches
            assert slabs >= 3
            assert called.downloads - before.downloads == slabs * len(outs)
            assert called.download_bytes - before.download_bytes == interior_bytes
            assert after.downloads == called.downloads
        ref = api.advection_step({"U": ins[0], "V": ins[1], "W": ins[2]}, geo.dx, geo.dy, geo.dz, geo.halo, ins[3:])
        for got, name in zip(outs, ["U", "V", "W", "S0"]):
            assert _same(got[geo.interior()], ref[name][geo.interior()])
    stats = dom.stats()
    dom.end_epoch()
    if path == "in place":
        # only the first two steps moved field data through copies
        assert stats.upload_bytes <= 2 * sum(a.nbytes for a in ins)


@pytest.mark.parametrize("nx, ny, nz", [(96, 64, 16), (512, 512, 24)])
def test_arrays_the_caller_page_locked_are_used_as_they_are(resident, cuda, nx, ny, nz):
    """Host arrays in memory the caller already page-locked (cudaHostAlloc, here through torch) are taken as
    pinned without a second registration, streamed like the runtime's own pinned arrays, and stay usable (and
    page-locked) after the domain closes."""
    dom, fns = resident
    geo = wl.Geometry(nx, ny, nz, halo=2)
    f = wl.advection_fields(geo, seed=9, nscalar=1)
    keep = [cuda.empty(a.shape, dtype=cuda.float64).pin_memory() for a in f.arrays() * 2]
    ins, outs = [t.numpy() for t in keep[:4]], [t.numpy() for t in keep[4:]]
    for a, src in zip(ins, f.arrays()):
        a[...] = src
    for a in outs:
        a[...] = 0.0
    dom.begin_epoch()
    h_in = [dom.bind_real64(a) for a in ins]
    h_out = [dom.bind_real64(a) for a in outs]
    arrays = [*h_out[:3], *h_in[:3], h_in[3], h_out[3]]
    for step in range(4):
        dom.host_modify(h_in)
        for a, src in zip(ins, f.arrays()):
            a[...] = src * (1.0 + 0.5 * step)
        assert _call(fns, dom, "advection::step1", arrays, [geo.dx, geo.dy, geo.dz],
                     [geo.nx, geo.ny, geo.nz, geo.halo]) == abi.OK
        dom.observe(h_out)
        ref = api.advection_step({"U": ins[0], "V": ins[1], "W": ins[2]}, geo.dx, geo.dy, geo.dz, geo.halo, ins[3:])
        for got, name in zip(outs, ["U", "V", "W", "S0"]):
            assert _same(got[geo.interior()], ref[name][geo.interior()])
    dom.end_epoch()
    dom.close()
    assert all(t.is_pinned() for t in keep)
    dev = keep[0].cuda(non_blocking=True)  # still page-locked: an asynchronous copy from it works
    cuda.cuda.synchronize()
    assert _same(dev.cpu().numpy(), ins[0])


@pytest.mark.parametrize("use, visible", [("host", None), ("host", ""), ("zero", None), ("device", None)])
def test_the_product_runtime_brings_the_device_up_only_for_device_work(use, visible, tmp_path):
    """The CUDA build: host-only use of 2 MiB arrays creates no stream and pins nothing, also with every device
    hidden; a device access brings the device up once (reference: test_scoped_runtime_cuda.py:404-410)."""
    import os
    import subprocess
    import sys

    from test_runtime_abi import HOST_ONLY

    assert native.LIBRARY.exists()
    script = tmp_path / "host_only.py"
    script.write_text(HOST_ONLY)
    env = {**os.environ, "FORT_RUNTIME_TRACE": "1"}
    if visible is not None:
        env["CUDA_VISIBLE_DEVICES"] = visible
    run = subprocess.run([sys.executable, str(script), str(native.LIBRARY), use, str(native.PACKAGE_ROOT)],
                         capture_output=True, text=True, timeout=120, env=env)
    assert run.returncode == 0, run.stdout + run.stderr
    initialized = [line for line in run.stderr.splitlines() if line.startswith("FORT_SCOPED initialize")]
    assert len(initialized) == (use == "device")
