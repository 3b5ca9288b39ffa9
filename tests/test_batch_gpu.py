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
