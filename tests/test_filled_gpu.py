"""The filled advance (F2C_ADVANCE_FILLED): one launch equals an advance step followed by the boundary fill,
over every cell of the padded arrays, bit for bit, for every kernel, single and batched."""

import numpy as np
import pytest

from compiler import native
from compiler import workloads as wl

pytestmark = pytest.mark.gpu

SHAPES = [(24, 20, 8, 2), (37, 19, 5, 2), (2, 3, 3, 2), (64, 64, 32, 1), (9, 33, 4, 3)]


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def _fields(torch, nx, ny, nz, h, nscalar, seed):
    geo = wl.Geometry(nx, ny, nz, halo=h)
    f = wl.advection_fields(geo, seed=seed, nscalar=nscalar)
    ins = [torch.from_numpy(a).cuda() for a in f.arrays()]
    grid = native.make_grid(nx, ny, nz, h, geo.dx, geo.dy, geo.dz)
    return geo, ins, grid


def _two_launches(torch, grid, ins, variant, nscalar):
    outs = [torch.full_like(t, float("nan")) for t in ins]
    p, q = [t.data_ptr() for t in ins], [t.data_ptr() for t in outs]
    native.advection(grid, *p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:], mode=native.ADVANCE, dt=0.1,
                     variant=variant)
    native.halo_fill(grid, q, [0, 0, 1] + [0] * nscalar)
    return outs


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("variant", [native.FACES, native.FAST, native.DIRECT])
def test_filled_advance_equals_advance_and_fill(cuda, shape, variant):
    nscalar = 2
    geo, ins, grid = _fields(cuda, *shape, nscalar, seed=sum(shape))
    want = _two_launches(cuda, grid, ins, variant, nscalar)
    got = [cuda.full_like(t, float("nan")) for t in ins]
    p, q = [t.data_ptr() for t in ins], [t.data_ptr() for t in got]
    native.advection(grid, *p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:], mode=native.ADVANCE_FILLED, dt=0.1,
                     variant=variant)
    cuda.cuda.synchronize()
    for n, (a, b) in enumerate(zip(got, want)):
        assert np.array_equal(_bits(a.cpu().numpy()), _bits(b.cpu().numpy())), (shape, n)


def test_filled_advance_keeps_pitch_padding(cuda):
    """A pitched grid: the cells beyond the padded rows and planes are never written."""
    nx, ny, nz, h = 20, 12, 6, 2
    sx, sy = nx + 2 * h + 5, ny + 2 * h + 3
    geo = wl.Geometry(nx, ny, nz, halo=h)
    f = wl.advection_fields(geo, seed=4, nscalar=0)
    grid = native.make_grid(nx, ny, nz, h, geo.dx, geo.dy, geo.dz, sx=sx, sy=sy)
    shape = (nz + 2 * h, sy, sx)

    def pitched(a):
        out = np.full(shape, np.nan)
        out[:, :ny + 2 * h, :nx + 2 * h] = a
        return cuda.from_numpy(out).cuda()

    ins = [pitched(a) for a in f.arrays()]
    want = _two_launches(cuda, grid, ins, native.FAST, 0)
    got = [cuda.full_like(t, float("nan")) for t in ins]
    p, q = [t.data_ptr() for t in ins], [t.data_ptr() for t in got]
    native.advection(grid, *p[:3], *q[:3], mode=native.ADVANCE_FILLED, dt=0.1, variant=native.FAST)
    cuda.cuda.synchronize()
    for a, b in zip(got, want):
        a, b = a.cpu().numpy(), b.cpu().numpy()
        assert np.isnan(a[:, ny + 2 * h:, :]).all() and np.isnan(a[:, :, nx + 2 * h:]).all()
        assert np.array_equal(_bits(a), _bits(b))


@pytest.mark.parametrize("rows,fast", [(8, False), (4, True), (8, True), (16, True)])
def test_filled_batch_equals_single_advance_and_fill(cuda, rows, fast):
    nscalar = 1
    inst = []
    for n, shape in enumerate(SHAPES):
        geo, ins, grid = _fields(cuda, *shape, nscalar, seed=40 + n)
        outs = [cuda.full_like(t, float("nan")) for t in ins]
        p, q = [t.data_ptr() for t in ins], [t.data_ptr() for t in outs]
        fields = native.make_fields(*p[:3], *q[:3], scalars=p[3:], scalar_out=q[3:], mode=native.ADVANCE_FILLED,
                                    dt=0.1)
        inst.append((grid, ins, outs, fields))
    batch = native.Batch([x[0] for x in inst], [x[3] for x in inst], kz=[3, 5, 2, 32, 4], tile_rows=rows)
    ws = cuda.empty(batch.workspace_bytes(), dtype=cuda.uint8, device="cuda")
    batch.prepare(ws.data_ptr(), ws.numel())
    batch.set_fast_fp(fast)
    batch.graph_step()
    cuda.cuda.synchronize()
    for grid, ins, outs, _ in inst:
        want = _two_launches(cuda, grid, ins, native.FAST if fast else native.FACES, nscalar)
        cuda.cuda.synchronize()
        for a, b in zip(outs, want):
            assert np.array_equal(_bits(a.cpu().numpy()), _bits(b.cpu().numpy()))


def test_filled_advance_refusals(cuda):
    geo, ins, grid = _fields(cuda, 16, 16, 8, 2, 0, seed=1)
    out = [cuda.empty_like(t) for t in ins]
    p, q = [t.data_ptr() for t in ins], [t.data_ptr() for t in out]
    with pytest.raises(native.NativeError, match="U, V and W"):
        native.advection(grid, *p[:3], q[0], q[1], None, mode=native.ADVANCE_FILLED, dt=0.1)
    flat = native.make_grid(16, 16, 2, 2, 1.0, 1.0, 1.0)
    with pytest.raises(native.NativeError, match="nz > halo"):
        native.advection(flat, *p[:3], *q[:3], mode=native.ADVANCE_FILLED, dt=0.1)
