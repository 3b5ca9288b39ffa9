"""Guard bands: no kernel writes outside what it owns.

compute-sanitizer is not available, so out-of-bounds writes are caught this
way: every array lives inside a larger allocation whose guard regions before
and after it, the unused tail of each padded row (x pitch) and the unused rows
of each padded plane (y pitch) hold a sentinel bit pattern. After the kernels
run, every sentinel outside the region a kernel may write must be unchanged,
and inputs must be unchanged entirely. Odd pitches and odd extents are used so
that no launch shape divides the arrays evenly.
"""

import ctypes as c

import numpy as np
import pytest

from compiler import native

pytestmark = pytest.mark.gpu

SENTINEL = np.array([0x7FF4DEADBEEF0001], dtype=np.uint64).view(np.float64)[0]  # a NaN no kernel produces
GUARD = 1031  # elements before and after each array


class Guarded:
    """A padded 3-D array (x pitch sx, y pitch sy) inside a sentinel-filled allocation.

    ``nz=None`` makes a single plane (a 2-D array with ghost rows and columns only)."""

    def __init__(self, torch, nx, ny, nz, h, sx, sy):
        self.torch = torch
        self.ex, self.ey = nx + 2 * h, ny + 2 * h
        self.ez = 1 if nz is None else nz + 2 * h
        self.sx, self.sy = sx, sy
        self.n = sx * sy * self.ez
        self.buf = torch.empty((self.n + 2 * GUARD,), dtype=torch.float64, device="cuda")
        self.buf.view(torch.int64).fill_(int(np.array([SENTINEL]).view(np.int64)[0]))
        self.ptr = self.buf.data_ptr() + 8 * GUARD

    def view(self, host):
        """(ez, sy, sx) view of the array part of a host copy of the allocation."""
        return host[GUARD:GUARD + self.n].reshape(self.ez, self.sy, self.sx)

    def host(self):
        return self.buf.cpu().numpy()

    def set_padded(self, values):
        """Write (ez, ey, ex) values into the padded layout (pads keep the sentinel)."""
        host = self.host()
        self.view(host)[:, :self.ey, :self.ex] = values
        self.buf.copy_(self.torch.from_numpy(host))

    def owned(self):
        """Mask over the allocation of the array's (ez, ey, ex) cells."""
        mask = np.zeros(self.n + 2 * GUARD, dtype=bool)
        self.view(mask)[:, :self.ey, :self.ex] = True
        return mask


def _sentinel_bits(a):
    return np.ascontiguousarray(a).view(np.uint64) == np.array([SENTINEL]).view(np.uint64)[0]


def _check(arr, before, writable):
    """Everything outside `writable` (a mask over the allocation) is bit-identical to `before`."""
    after = arr.host()
    keep = ~writable
    assert np.array_equal(after[keep].view(np.uint64), before[keep].view(np.uint64))


def _interior_mask(arr, h):
    mask = np.zeros(arr.n + 2 * GUARD, dtype=bool)
    v = arr.view(mask)
    v[h:arr.ez - h, h:arr.ey - h, h:arr.ex - h] = True
    return mask


def _fields(torch, nx, ny, nz, h, sx, sy, count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for n in range(count):
        g = Guarded(torch, nx, ny, nz, h, sx, sy)
        g.set_padded(rng.random((nz + 2 * h, ny + 2 * h, nx + 2 * h)) * 2.0 - 1.0)
        out.append(g)
    return out


@pytest.mark.parametrize("mode", [native.TENDENCY, native.ADVANCE])
def test_advection_writes_only_output_interiors(cuda, mode):
    nx, ny, nz, h = 45, 19, 13, 2
    sx, sy = nx + 2 * h + 3, ny + 2 * h + 2
    ins = _fields(cuda, nx, ny, nz, h, sx, sy, 5, seed=1)                   # U, V, W, two scalars
    outs = [Guarded(cuda, nx, ny, nz, h, sx, sy) for _ in range(5)]
    before_in = [a.host() for a in ins]
    before_out = [a.host() for a in outs]
    grid = native.make_grid(nx, ny, nz, h, 10.0, 10.0, 5.0, sx, sy)
    native.advection(grid, *[a.ptr for a in ins[:3]], *[a.ptr for a in outs[:3]],
                     scalars=[a.ptr for a in ins[3:]], scalar_out=[a.ptr for a in outs[3:]], mode=mode, dt=0.1)
    cuda.cuda.synchronize()
    for a, b in zip(ins, before_in):
        _check(a, b, np.zeros(a.n + 2 * GUARD, dtype=bool))
    for a, b in zip(outs, before_out):
        inner = _interior_mask(a, h)
        _check(a, b, inner)
        assert not _sentinel_bits(a.host()[inner]).any()  # and the interior was written


def test_halo_fill_writes_only_ghosts(cuda):
    nx, ny, nz, h = 33, 17, 9, 2
    sx, sy = nx + 2 * h + 5, ny + 2 * h + 1
    fields = _fields(cuda, nx, ny, nz, h, sx, sy, 4, seed=2)
    before = [a.host() for a in fields]
    grid = native.make_grid(nx, ny, nz, h, 1.0, 1.0, 1.0, sx, sy)
    native.halo_fill(grid, [a.ptr for a in fields], [0, 0, 1, 0])
    cuda.cuda.synchronize()
    for n, (a, b) in enumerate(zip(fields, before)):
        ghosts = a.owned() & ~_interior_mask(a, h)
        if n == 2:  # W: the top wall level h+nz-1 is set to zero as well
            a.view(ghosts)[h + nz - 1, h:h + ny, h:h + nx] = True
        _check(a, b, ghosts)


def test_batched_step_and_halo_stay_inside_their_instances(cuda):
    shapes = [(37, 11, 7), (8, 21, 12), (64, 9, 5)]
    h = 2
    insts, befores = [], []
    grids, fields = [], []
    for n, (nx, ny, nz) in enumerate(shapes):
        sx, sy = nx + 2 * h + 1 + n, ny + 2 * h + 2
        ins = _fields(cuda, nx, ny, nz, h, sx, sy, 4, seed=10 + n)
        outs = [Guarded(cuda, nx, ny, nz, h, sx, sy) for _ in range(4)]
        insts.append((ins, outs))
        befores.append(([a.host() for a in ins], [a.host() for a in outs]))
        grids.append(native.make_grid(nx, ny, nz, h, 10.0, 10.0, 5.0, sx, sy))
        fields.append(native.make_fields(*[a.ptr for a in ins[:3]], *[a.ptr for a in outs[:3]],
                                         scalars=[ins[3].ptr], scalar_out=[outs[3].ptr], mode=native.ADVANCE, dt=0.1))
    batch = native.Batch(grids, fields, kz=[3, 5, 2])
    ws = cuda.empty(batch.workspace_bytes(), dtype=cuda.uint8, device="cuda")
    batch.prepare(ws.data_ptr(), ws.numel())
    batch.step()
    batch.halo()
    cuda.cuda.synchronize()
    for (ins, outs), (bin_, bout) in zip(insts, befores):
        for a, b in zip(ins, bin_):
            _check(a, b, np.zeros(a.n + 2 * GUARD, dtype=bool))
        for a, b in zip(outs, bout):
            _check(a, b, a.owned())                       # the step writes interiors, the fill the ghosts
            assert not _sentinel_bits(a.host()[a.owned()]).any()


def test_stencils_write_only_their_outputs_interior(cuda):
    lib = native.load()
    lib.f2c_diffusion7_v1.argtypes = [c.POINTER(native.Grid), c.c_void_p, c.c_void_p, c.c_double, c.c_double,
                                      c.c_void_p]
    lib.f2c_jacobi5_v1.argtypes = [c.c_void_p, c.c_void_p, c.c_int64, c.c_int64, c.c_int64, c.c_int64, c.c_void_p]
    lib.f2c_yee2d_v1.argtypes = [c.c_void_p] * 3 + [c.c_int64] * 4 + [c.c_double, c.c_double, c.c_void_p]
    # diffusion, 3-D, pitched
    nx, ny, nz, h = 29, 14, 11, 1
    sx, sy = nx + 2 * h + 3, ny + 2 * h + 1
    (a,) = _fields(cuda, nx, ny, nz, h, sx, sy, 1, seed=20)
    b = Guarded(cuda, nx, ny, nz, h, sx, sy)
    ba, bb = a.host(), b.host()
    grid = native.make_grid(nx, ny, nz, h, 1.0, 1.0, 1.0, sx, sy)
    assert lib.f2c_diffusion7_v1(c.byref(grid), a.ptr, b.ptr, 0.1, 1.0, None) == 0
    cuda.cuda.synchronize()
    _check(a, ba, np.zeros(a.n + 2 * GUARD, dtype=bool))
    _check(b, bb, _interior_mask(b, h))
    # Jacobi and Yee: single planes with a row pitch
    nx, ny, h = 37, 23, 1
    sx = nx + 2 * h + 5
    rng = np.random.default_rng(22)

    def plane():
        g = Guarded(cuda, nx, ny, None, h, sx, ny + 2 * h)
        g.set_padded(rng.random((1, ny + 2 * h, nx + 2 * h)))
        return g

    u, v = plane(), Guarded(cuda, nx, ny, None, h, sx, ny + 2 * h)
    bu, bv = u.host(), v.host()
    assert lib.f2c_jacobi5_v1(u.ptr, v.ptr, nx, ny, h, sx, None) == 0
    cuda.cuda.synchronize()
    _check(u, bu, np.zeros(u.n + 2 * GUARD, dtype=bool))
    inner = np.zeros(v.n + 2 * GUARD, dtype=bool)
    v.view(inner)[0, h:ny + h, h:nx + h] = True
    _check(v, bv, inner)
    ez, hx, hy = plane(), plane(), plane()
    before = [x.host() for x in (ez, hx, hy)]
    assert lib.f2c_yee2d_v1(ez.ptr, hx.ptr, hy.ptr, nx, ny, h, sx, 0.1, 0.2, None) == 0
    cuda.cuda.synchronize()
    for x, bx in zip((ez, hx, hy), before):
        m = np.zeros(x.n + 2 * GUARD, dtype=bool)
        x.view(m)[0, h:ny + h, h:nx + h] = True
        _check(x, bx, m)
