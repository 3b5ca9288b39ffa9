"""Batched ensembles: one persistent launch over a tile queue equals one launch per instance, bit for bit."""

import numpy as np
import pytest

from compiler import native
from compiler import workloads as wl
from oracle import api

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


SHAPES = [(64, 32, 20), (37, 19, 33), (96, 64, 12), (8, 9, 70), (130, 17, 5)]


def _setup(torch, nscalar, mode=native.TENDENCY, dt=0.0):
    inst = []
    for n, (nx, ny, nz) in enumerate(SHAPES):
        geo = wl.Geometry(nx, ny, nz, halo=2)
        f = wl.advection_fields(geo, seed=100 + n, nscalar=nscalar)
        ins = [torch.from_numpy(a).cuda() for a in f.arrays()]
        outs = [torch.full_like(t, float("nan")) for t in ins]
        grid = native.make_grid(nx, ny, nz, 2, geo.dx, geo.dy, geo.dz)
        p = [t.data_ptr() for t in ins]
        q = [t.data_ptr() for t in outs]
        fields = native.make_fields(*p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:], mode=mode, dt=dt)
        inst.append((geo, f, ins, outs, grid, fields))
    return inst


@pytest.mark.parametrize("nscalar,kz", [(1, None), (0, [8, 16, 12, 32, 5]), (3, [64] * 5)])
def test_batch_matches_oracle(cuda, nscalar, kz):
    inst = _setup(cuda, nscalar)
    batch = native.Batch([x[4] for x in inst], [x[5] for x in inst], kz=kz)
    ws = cuda.empty(batch.workspace_bytes(), dtype=cuda.uint8, device="cuda")
    batch.prepare(ws.data_ptr(), ws.numel())
    for _ in range(2):  # the counter is reset by every step
        batch.step()
    cuda.cuda.synchronize()
    for geo, f, ins, outs, grid, fields in inst:
        ref = api.advection_step({"U": f.U, "V": f.V, "W": f.W}, geo.dx, geo.dy, geo.dz, geo.halo, f.scalars)
        names = ["U", "V", "W", *[f"S{n}" for n in range(nscalar)]]
        for got, name in zip(outs, names):
            g = got.cpu().numpy()
            assert np.array_equal(_bits(g[geo.interior()]), _bits(ref[name][geo.interior()]))
            ghost = g.copy()
            ghost[geo.interior()] = 0.0
            assert np.isnan(ghost[np.ones_like(ghost, dtype=bool) & (ghost != 0.0)]).all()


def test_batch_advance_mode_equals_single_launches(cuda):
    inst = _setup(cuda, 1, mode=native.ADVANCE, dt=0.1)
    batch = native.Batch([x[4] for x in inst], [x[5] for x in inst])
    ws = cuda.empty(batch.workspace_bytes(), dtype=cuda.uint8, device="cuda")
    batch.prepare(ws.data_ptr(), ws.numel())
    batch.step()
    cuda.cuda.synchronize()
    for geo, f, ins, outs, grid, fields in inst:
        single = [cuda.full_like(t, float("nan")) for t in ins]
        q = [t.data_ptr() for t in single]
        p = [t.data_ptr() for t in ins]
        native.advection(grid, *p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:], mode=native.ADVANCE, dt=0.1)
        cuda.cuda.synchronize()
        for a, b in zip(outs, single):
            assert np.array_equal(_bits(a.cpu().numpy()[geo.interior()]), _bits(b.cpu().numpy()[geo.interior()]))


def test_batch_rejects_mixed_instances(cuda):
    inst = _setup(cuda, 1)
    fields = [x[5] for x in inst]
    fields[1].nscalar = 0
    batch = native.Batch([x[4] for x in inst], fields)
    ws = cuda.empty(batch.workspace_bytes(), dtype=cuda.uint8, device="cuda")
    with pytest.raises(native.NativeError):
        batch.prepare(ws.data_ptr(), ws.numel())
    with pytest.raises(native.NativeError):
        native.Batch([x[4] for x in inst], [x[5] for x in inst]).prepare(ws.data_ptr(), 64)


def test_async_prepare_and_batched_halo_equal_the_single_instance_path(cuda):
    """prepare_async (through pinned staging) plans what prepare does, and one batched boundary fill writes
    every instance's ghosts exactly as one f2c_halo_fill_v1 per instance."""
    nscalar = 2
    inst = _setup(cuda, nscalar, mode=native.ADVANCE, dt=0.1)
    ref = _setup(cuda, nscalar, mode=native.ADVANCE, dt=0.1)
    batch = native.Batch([x[4] for x in inst], [x[5] for x in inst])
    ws = cuda.empty(batch.workspace_bytes(), dtype=cuda.uint8, device="cuda")
    staging = cuda.empty(batch.workspace_bytes(), dtype=cuda.uint8, pin_memory=True)
    stream = cuda.cuda.Stream()
    batch.prepare_async(ws.data_ptr(), ws.numel(), staging.data_ptr(), stream.cuda_stream)
    batch.step(stream.cuda_stream)
    batch.halo(stream.cuda_stream)
    stream.synchronize()
    single = native.Batch([x[4] for x in ref], [x[5] for x in ref])
    ws2 = cuda.empty(single.workspace_bytes(), dtype=cuda.uint8, device="cuda")
    single.prepare(ws2.data_ptr(), ws2.numel())
    assert (batch.plan.items, batch.plan.ctas, batch.plan.count) == (single.plan.items, single.plan.ctas,
                                                                     single.plan.count)
    single.step()
    for geo, f, ins, outs, grid, fields in ref:
        native.halo_fill(grid, [t.data_ptr() for t in outs], [0, 0, 1] + [0] * nscalar)
    cuda.cuda.synchronize()
    for a, b in zip(inst, ref):
        for x, y in zip(a[3], b[3]):
            assert np.array_equal(_bits(x.cpu().numpy()), _bits(y.cpu().numpy()))


def test_batched_halo_refuses_instances_too_small_for_the_fill(cuda):
    geo = wl.Geometry(16, 16, 2, halo=2)  # nz must exceed the halo
    f = wl.advection_fields(geo, seed=1, nscalar=0)
    ins = [cuda.from_numpy(a).cuda() for a in f.arrays()]
    outs = [cuda.zeros_like(t) for t in ins]
    grid = native.make_grid(16, 16, 2, 2, geo.dx, geo.dy, geo.dz)
    fields = native.make_fields(*[t.data_ptr() for t in ins], *[t.data_ptr() for t in outs], mode=native.ADVANCE,
                                dt=0.1)
    batch = native.Batch([grid], [fields])
    ws = cuda.empty(batch.workspace_bytes(), dtype=cuda.uint8, device="cuda")
    batch.prepare(ws.data_ptr(), ws.numel())
    with pytest.raises(native.NativeError, match="halo fill needs"):
        batch.halo()


def test_fast_batch_on_the_ensemble_shapes(cuda):
    """The 64-instance ensemble (nx, ny from {64..256}, nz from {32, 64, 96}, seed 1; U, V, W + 1 scalar) stepped
    by the fast-fp persistent kernel: every instance within the fast-fp tolerance of the oracle, and bit-identical
    to the fast kernel launched on each instance alone (the same tile arithmetic)."""
    import tolerance

    shapes = wl.ensemble_shapes(64, seed=1)
    inst = []
    for n, (nx, ny, nz) in enumerate(shapes):
        geo = wl.Geometry(nx, ny, nz, halo=2)
        f = wl.advection_fields(geo, seed=1000 + n, nscalar=1)
        ins = [cuda.from_numpy(a).cuda() for a in f.arrays()]
        outs = [cuda.full_like(t, float("nan")) for t in ins]
        grid = native.make_grid(nx, ny, nz, 2, geo.dx, geo.dy, geo.dz)
        p, q = [t.data_ptr() for t in ins], [t.data_ptr() for t in outs]
        inst.append((geo, f, ins, outs, grid, native.make_fields(*p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:])))
    batch = native.Batch([x[4] for x in inst], [x[5] for x in inst])
    ws = cuda.empty(batch.workspace_bytes(), dtype=cuda.uint8, device="cuda")
    batch.prepare(ws.data_ptr(), ws.numel())
    batch.set_fast_fp()
    batch.step()
    cuda.cuda.synchronize()
    for geo, f, ins, outs, grid, fields in inst:
        alone = [cuda.full_like(t, float("nan")) for t in ins]
        p, q = [t.data_ptr() for t in ins], [t.data_ptr() for t in alone]
        native.advection(grid, *p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:], variant=native.FAST)
        ref = api.advection_step({"U": f.U, "V": f.V, "W": f.W}, geo.dx, geo.dy, geo.dz, geo.halo, f.scalars)
        inner = geo.interior()
        for got, one, name in zip(outs, alone, ["U", "V", "W", "S0"]):
            g = got.cpu().numpy()[inner]
            assert np.array_equal(_bits(g), _bits(one.cpu().numpy()[inner])), name
            tolerance.check(g, ref[name][inner], name)


@pytest.mark.parametrize("rows", [4, 8, 16])
@pytest.mark.parametrize("kz", [None, [3, 7, 32, 16, 2]])
def test_fast_batch_tile_shapes_equal_single_launches(cuda, rows, kz):
    """Every tile height and chunk depth gives the single-instance fast-fp kernel's values bit for bit, and the
    oracle's within the fast-fp tolerance; the batch's own graph replays the same step."""
    from tolerance import check

    inst = _setup(cuda, 2)
    batch = native.Batch([x[4] for x in inst], [x[5] for x in inst], kz=kz, tile_rows=rows)
    ws = cuda.empty(batch.workspace_bytes(), dtype=cuda.uint8, device="cuda")
    batch.prepare(ws.data_ptr(), ws.numel())
    if rows != 8:
        assert batch.plan.reserved & native.BATCH_FAST_FP  # set by preparation: only the fast-fp kernel has them
    else:
        batch.set_fast_fp(True)
    assert (batch.plan.reserved >> 8) & 0xFF == rows
    for _ in range(2):
        batch.graph_step()
    cuda.cuda.synchronize()
    for geo, f, ins, outs, grid, fields in inst:
        single = [cuda.full_like(t, float("nan")) for t in ins]
        p, q = [t.data_ptr() for t in ins], [t.data_ptr() for t in single]
        native.advection(grid, *p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:], variant=native.FAST)
        cuda.cuda.synchronize()
        ref = api.advection_step({"U": f.U, "V": f.V, "W": f.W}, geo.dx, geo.dy, geo.dz, geo.halo, f.scalars)
        for got, one, name in zip(outs, single, ["U", "V", "W", "S0", "S1"]):
            g = got.cpu().numpy()[geo.interior()]
            assert np.array_equal(_bits(g), _bits(one.cpu().numpy()[geo.interior()])), name
            check(g, ref[name][geo.interior()], name)


def test_strict_step_refuses_short_and_tall_tiles(cuda):
    inst = _setup(cuda, 0)
    batch = native.Batch([x[4] for x in inst], [x[5] for x in inst], tile_rows=16)
    ws = cuda.empty(batch.workspace_bytes(), dtype=cuda.uint8, device="cuda")
    batch.prepare(ws.data_ptr(), ws.numel())
    batch.set_fast_fp(False)
    with pytest.raises(native.NativeError, match="fast-fp"):
        batch.step()
    with pytest.raises(native.NativeError, match="tile rows"):
        native.Batch([x[4] for x in inst], [x[5] for x in inst], tile_rows=12).prepare(ws.data_ptr(), ws.numel())


def test_batch_rejects_an_instance_too_wide_for_the_tile_queue(cuda):
    """Item tile indices are 16-bit: an instance wider than 32767 tiles is refused before any device work (the
    field pointers below are never dereferenced)."""
    wide = native.make_grid(32767 * 32 + 1, 8, 4, 2, 1.0, 1.0, 1.0)
    fake = 256
    fields = native.make_fields(fake, fake, fake, fake, fake, fake)
    batch = native.Batch([wide], [fields])
    with pytest.raises(native.NativeError, match="too wide"):
        batch.prepare(fake, 1 << 30)
